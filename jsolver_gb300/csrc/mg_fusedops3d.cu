// mg_fusedops3d.cu — the 3D cycle's operators fused pairwise over shared-memory tiles with
// halos, for the grid-wide levels whose launches are bound by latency rather than bytes
// (up to 2^19 padded points: 64^3 and smaller above the coarse block). Opt-in
// (JMG_FUSEDOPS3D=1): measured no faster than the separate launches in the 3D solves.
//
//   k_smooth_restrict3d   the last pre-smoothing sweep (red then black,
//                         solver_3d.py:679-706) followed by the defect and restriction onto
//                         the next level (solver_3d.py:622-652), which also zeroes phi_c;
//   k_prolong_smooth3d    the prolongation phi += P phi_c (solver_3d.py:618, 654-677)
//                         followed by the first post-smoothing sweep.
//
// The same scheme as the 2D pairs (mg_fusedops2d.cuh), in three dimensions. A tile
// recomputes everything its outputs depend on from the level's arrays, so no block reads
// what another writes: the smoothed phi goes to the level's second buffer and the two
// buffers swap (twice per visit).
//
// Smooth + restrict, per block a CZ x CY x CX tile of coarse points. The coarse point
// (K, J, I) restricts the 13 red defects around fine (2K-1, 2J-1, 2I-1); the fine footprint
// runs from 2K0-2 to 2K0+2CZ-2 per axis. The defects read black values after the sweep on
// the footprint plus one; those read red values on the footprint plus two; those read old
// phi on the footprint plus three. The block owns fine 2K0-1 .. 2K0+2CZ-2 per axis.
//
// Prolong + smooth, per block a TZ x TY x TX tile of fine interior points. Black values of
// the tile read red values on the tile plus one; those read prolongated black values (old
// phi + the class's interpolation) on the tile plus two. Black points are those with one
// or three even indices, whose interpolation the reference always applies; red points are
// overwritten by the red pass without being read (the reference's bilinear class is red
// and skipped when nu2 > 0).
//
// Red is the colour with i+j+k odd (solver_3d.py:693). Every value is computed with
// gs_point3d's / defect_point3d's / restrict_point3d's / prolong_point3d's arithmetic in
// the same order, so solves give the same bits as the unfused operators (the default;
// tests/test_gpu_fused.py compares).
#include <cstdlib>

#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

constexpr int kNT = 512;

template <typename T, int CZ, int CY, int CX>
struct SR3 {
  static constexpr int DZ = 2 * CZ + 1, DY = 2 * CY + 1, DX = 2 * CX + 1;  // footprint (red defects)
  static constexpr int NZ = DZ + 4, NY = DY + 4, NX = DX + 4;              // new phi: footprint + 2
  static constexpr int OZ = DZ + 6, OY = DY + 6, OX = DX + 6;              // old phi: footprint + 3
  static constexpr size_t smem = sizeof(T) * ((size_t)OZ * OY * OX + (size_t)NZ * NY * NX + (size_t)DZ * DY * DX);
};

template <typename T, int TZ, int TY, int TX>
struct PS3 {
  static constexpr int BZ = TZ + 4, BY = TY + 4, BX = TX + 4;  // prolongated black values: tile + 2
  static constexpr int RZ = TZ + 2, RY = TY + 2, RX = TX + 2;  // new red values: tile + 1
  static constexpr size_t smem = sizeof(T) * ((size_t)BZ * BY * BX + (size_t)RZ * RY * RX);
};

// tile shapes: 4 x 4 x 8 coarse points for smooth + restrict (FP32 40 KB, FP64 81 KB of
// shared memory) and 4 x 8 x 16 fine points for prolong + smooth (12 / 24 KB)
constexpr int kCZ = 4, kCY = 4, kCX = 8;
constexpr int kTZ = 4, kTY = 8, kTX = 16;

__device__ __forceinline__ bool interior(int k, int j, int i, const int mz, const int my, const int mx) {
  return k >= 2 && k <= mz && j >= 2 && j <= my && i >= 2 && i <= mx;
}

template <typename T, int CZ, int CY, int CX>
__global__ void __launch_bounds__(kNT) k_smooth_restrict3d(Lvl<T> f, T* __restrict__ out, Lvl<T> c, int zero_in) {
  pdl_enter();
  using G = SR3<T, CZ, CY, CX>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* Old = reinterpret_cast<T*>(smraw);  // [OZ][OY][OX], fine (fz0 - 3 + z, fy0 - 3 + y, fx0 - 3 + x)
  T* New = Old + G::OZ * G::OY * G::OX;  // [NZ][NY][NX], fine (fz0 - 2 + z, ...)
  T* Def = New + G::NZ * G::NY * G::NX;  // [DZ][DY][DX], fine (fz0 + z, ...)
  const int K0 = blockIdx.z * CZ, J0 = blockIdx.y * CY, I0 = blockIdx.x * CX;
  const int fz0 = 2 * K0 - 2, fy0 = 2 * J0 - 2, fx0 = 2 * I0 - 2;
  const int tid = threadIdx.x;
  const long long P = f.P, S = f.S;
  const int mx = f.mx, my = f.my, mz = f.mz;
  constexpr int OYX = G::OY * G::OX, NYX = G::NY * G::NX, DYX = G::DY * G::DX;
  // 1. old phi (zero outside the padded array; not read from a zero initial guess)
  if (!zero_in) {
    for (int t = tid; t < G::OZ * OYX; t += kNT) {
      const int z = t / OYX, r = t - z * OYX, y = r / G::OX, x = r - y * G::OX;
      const int k = fz0 - 3 + z, j = fy0 - 3 + y, i = fx0 - 3 + x;
      T v = T(0);
      if (k >= 0 && j >= 0 && i >= 0 && k <= mz + 2 && j <= my + 2 && i <= mx + 2) v = f.phi[k * S + j * P + i];
      Old[t] = v;
    }
  }
  __syncthreads();
  // 2. red pass (i + j + k odd) on the footprint + 2; non-interior points stay zero
  {
    constexpr int XR = (G::NX + 1) / 2, N = G::NZ * G::NY * XR;
    for (int t = tid; t < N; t += kNT) {
      const int z = t / (G::NY * XR), r = t - z * (G::NY * XR), y = r / XR, xp = r - y * XR;
      const int k = fz0 - 2 + z, j = fy0 - 2 + y;
      const int x = 2 * xp + ((1 - k - j - (fx0 - 2)) & 1);
      if (x >= G::NX) continue;
      const int i = fx0 - 2 + x;
      const int slot = (z * G::NY + y) * G::NX + x;
      if (!interior(k, j, i, mz, my, mx)) {
        New[slot] = T(0);
        continue;
      }
      const long long p = k * S + j * P + i;
      T v;
      if (zero_in) {
        v = (T(0) - f.rhs[p]) * f.invd[p];
      } else {
        const T* o = Old + ((z + 1) * G::OY + (y + 1)) * G::OX + (x + 1);  // the same point in Old
        T s = f.wz[p] * o[OYX];
        s = fma(f.wz[p - S], o[-OYX], s);
        s = fma(f.wy[p], o[G::OX], s);
        s = fma(f.wy[p - P], o[-G::OX], s);
        s = fma(f.wx[p], o[1], s);
        s = fma(f.wx[p - 1], o[-1], s);
        s = s - f.rhs[p];
        v = s * f.invd[p];
      }
      New[slot] = v;
    }
  }
  __syncthreads();
  // 3. black pass (i + j + k even) on the footprint + 1 from the new red values
  {
    constexpr int BZ = G::DZ + 2, BY = G::DY + 2, BX = G::DX + 2;
    constexpr int XB = (BX + 1) / 2, N = BZ * BY * XB;
    for (int t = tid; t < N; t += kNT) {
      const int z = t / (BY * XB), r = t - z * (BY * XB), y = r / XB, xp = r - y * XB;
      const int k = fz0 - 1 + z, j = fy0 - 1 + y;
      const int x = 2 * xp + ((k + j + fx0 - 1) & 1);  // i = fx0 - 1 + x with i + j + k even
      if (x >= BX) continue;
      const int i = fx0 - 1 + x;
      const int slot = ((z + 1) * G::NY + (y + 1)) * G::NX + (x + 1);  // position in New
      if (!interior(k, j, i, mz, my, mx)) {
        New[slot] = T(0);
        continue;
      }
      const long long p = k * S + j * P + i;
      const T* n = New + slot;
      T s = f.wz[p] * n[NYX];
      s = fma(f.wz[p - S], n[-NYX], s);
      s = fma(f.wy[p], n[G::NX], s);
      s = fma(f.wy[p - P], n[-G::NX], s);
      s = fma(f.wx[p], n[1], s);
      s = fma(f.wx[p - 1], n[-1], s);
      s = s - f.rhs[p];
      New[slot] = s * f.invd[p];
    }
  }
  __syncthreads();
  // 4. red defects on the footprint (0 outside the interior); the owned smoothed phi out
  {
    constexpr int XR = (G::DX + 1) / 2, N = G::DZ * G::DY * XR;
    for (int t = tid; t < N; t += kNT) {
      const int z = t / (G::DY * XR), r = t - z * (G::DY * XR), y = r / XR, xp = r - y * XR;
      const int k = fz0 + z, j = fy0 + y;
      const int x = 2 * xp + ((1 - k - j - fx0) & 1);
      if (x >= G::DX) continue;
      const int i = fx0 + x;
      const int slot = (z * G::DY + y) * G::DX + x;
      if (!interior(k, j, i, mz, my, mx)) {
        Def[slot] = T(0);
        continue;
      }
      const long long p = k * S + j * P + i;
      const T* n = New + ((z + 2) * G::NY + (y + 2)) * G::NX + (x + 2);
      // defect_point3d's order
      T d = f.acc[p] * n[0];
      d = fma(-f.wx[p - 1], n[-1], d);
      d = fma(-f.wx[p], n[1], d);
      d = fma(-f.wy[p - P], n[-G::NX], d);
      d = fma(-f.wy[p], n[G::NX], d);
      d = fma(-f.wz[p - S], n[-NYX], d);
      d = fma(-f.wz[p], n[NYX], d);
      Def[slot] = d + f.rhs[p];
    }
    // owned fine points: fz0 + 1 .. fz0 + 2CZ per axis (interior ones)
    constexpr int OWZ = 2 * CZ, OWY = 2 * CY, OWX = 2 * CX;
    for (int t = tid; t < OWZ * OWY * OWX; t += kNT) {
      const int z = t / (OWY * OWX), r = t - z * (OWY * OWX), y = r / OWX, x = r - y * OWX;
      const int k = fz0 + 1 + z, j = fy0 + 1 + y, i = fx0 + 1 + x;
      if (interior(k, j, i, mz, my, mx)) out[k * S + j * P + i] = New[((z + 3) * G::NY + (y + 3)) * G::NX + (x + 3)];
    }
  }
  __syncthreads();
  // 5. coarse rhs (restrict_point3d's order) and phi_c = 0 over the padded coarse tile
  const long long Pc = c.P, Sc = c.S;
  for (int t = tid; t < CZ * CY * CX; t += kNT) {
    const int K = K0 + t / (CY * CX), J = J0 + (t / CX) % CY, I = I0 + t % CX;
    if (K > c.mz + 2 || J > c.my + 2 || I > c.mx + 2) continue;
    T v = T(0);
    if (interior(K, J, I, c.mz, c.my, c.mx)) {
      const T* d = Def + ((2 * K - 1 - fz0) * G::DY + (2 * J - 1 - fy0)) * G::DX + (2 * I - 1 - fx0);
      constexpr int PD = G::DX, SD = DYX;
      T s = d[PD + 1];
      s = s + d[PD - 1];
      s = s + d[-PD + 1];
      s = s + d[-PD - 1];
      s = s + d[SD + 1];
      s = s + d[SD - 1];
      s = s + d[-SD + 1];
      s = s + d[-SD - 1];
      s = s + d[SD + PD];
      s = s + d[SD - PD];
      s = s + d[-SD + PD];
      s = s + d[-SD - PD];
      v = T(0.03125) * s + T(0.125) * d[0];
    }
    c.rhs[K * Sc + J * Pc + I] = v;
    c.phi[K * Sc + J * Pc + I] = T(0);
  }
}

template <typename T, int TZ, int TY, int TX>
__global__ void __launch_bounds__(kNT) k_prolong_smooth3d(Lvl<T> f, T* __restrict__ out, Lvl<T> c) {
  pdl_enter();
  using G = PS3<T, TZ, TY, TX>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* Blk = reinterpret_cast<T*>(smraw);  // [BZ][BY][BX], fine (k0 - 2 + z, j0 - 2 + y, i0 - 2 + x)
  T* Red = Blk + G::BZ * G::BY * G::BX;  // [RZ][RY][RX], fine (k0 - 1 + z, ...)
  const int k0 = 2 + blockIdx.z * TZ, j0 = 2 + blockIdx.y * TY, i0 = 2 + blockIdx.x * TX;
  const int tid = threadIdx.x;
  const long long P = f.P, S = f.S;
  const int mx = f.mx, my = f.my, mz = f.mz;
  constexpr int BYX = G::BY * G::BX, RYX = G::RY * G::RX;
  // 1. black points (i + j + k even) of the tile + 2: old phi + the interpolated correction
  {
    constexpr int XB = (G::BX + 1) / 2, N = G::BZ * G::BY * XB;
    for (int t = tid; t < N; t += kNT) {
      const int z = t / (G::BY * XB), r = t - z * (G::BY * XB), y = r / XB, xp = r - y * XB;
      const int k = k0 - 2 + z, j = j0 - 2 + y;
      const int x = 2 * xp + ((k + j + i0 - 2) & 1);
      if (x >= G::BX) continue;
      const int i = i0 - 2 + x;
      const int slot = (z * G::BY + y) * G::BX + x;
      if (!interior(k, j, i, mz, my, mx)) {
        Blk[slot] = T(0);
        continue;
      }
      T corr = T(0);
      prolong_point3d<T>(c, k, j, i, true, &corr);  // one or three even indices: always applied
      Blk[slot] = f.phi[k * S + j * P + i] + corr;
    }
  }
  __syncthreads();
  // 2. red pass on the tile + 1
  {
    constexpr int XR = (G::RX + 1) / 2, N = G::RZ * G::RY * XR;
    for (int t = tid; t < N; t += kNT) {
      const int z = t / (G::RY * XR), r = t - z * (G::RY * XR), y = r / XR, xp = r - y * XR;
      const int k = k0 - 1 + z, j = j0 - 1 + y;
      const int x = 2 * xp + ((1 - k - j - (i0 - 1)) & 1);
      if (x >= G::RX) continue;
      const int i = i0 - 1 + x;
      const int slot = (z * G::RY + y) * G::RX + x;
      if (!interior(k, j, i, mz, my, mx)) {
        Red[slot] = T(0);
        continue;
      }
      const long long p = k * S + j * P + i;
      const T* b = Blk + ((z + 1) * G::BY + (y + 1)) * G::BX + (x + 1);
      T s = f.wz[p] * b[BYX];
      s = fma(f.wz[p - S], b[-BYX], s);
      s = fma(f.wy[p], b[G::BX], s);
      s = fma(f.wy[p - P], b[-G::BX], s);
      s = fma(f.wx[p], b[1], s);
      s = fma(f.wx[p - 1], b[-1], s);
      s = s - f.rhs[p];
      Red[slot] = s * f.invd[p];
    }
  }
  __syncthreads();
  // 3. black pass on the tile; both colours of the tile out
  {
    for (int t = tid; t < TZ * TY * TX; t += kNT) {
      const int z = t / (TY * TX), r = t - z * (TY * TX), y = r / TX, x = r - y * TX;
      const int k = k0 + z, j = j0 + y, i = i0 + x;
      if (k > mz || j > my || i > mx) continue;
      const long long p = k * S + j * P + i;
      const T* n = Red + ((z + 1) * G::RY + (y + 1)) * G::RX + (x + 1);
      if (((i + j + k) & 1) != 0) {  // red: the value of the red pass
        out[p] = n[0];
        continue;
      }
      T s = f.wz[p] * n[RYX];
      s = fma(f.wz[p - S], n[-RYX], s);
      s = fma(f.wy[p], n[G::RX], s);
      s = fma(f.wy[p - P], n[-G::RX], s);
      s = fma(f.wx[p], n[1], s);
      s = fma(f.wx[p - 1], n[-1], s);
      s = s - f.rhs[p];
      out[p] = s * f.invd[p];
    }
  }
}

template <typename T>
bool set_smem_attrs3() {
  static const bool ok = [] {
    const int a = (int)SR3<T, kCZ, kCY, kCX>::smem, b = (int)PS3<T, kTZ, kTY, kTX>::smem;
    return cudaFuncSetAttribute(k_smooth_restrict3d<T, kCZ, kCY, kCX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                a) == cudaSuccess &&
           cudaFuncSetAttribute(k_prolong_smooth3d<T, kTZ, kTY, kTX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                b) == cudaSuccess;
  }();
  return ok;
}

}  // namespace

template <typename T>
void launch_smooth_restrict3d(Lvl<T>& f, const Lvl<T>& c, bool zero_in, cudaStream_t s) {
  set_smem_attrs3<T>();
  dim3 g((unsigned)((c.mx + 3 + kCX - 1) / kCX), (unsigned)((c.my + 3 + kCY - 1) / kCY),
         (unsigned)((c.mz + 3 + kCZ - 1) / kCZ));
  launch_k(k_smooth_restrict3d<T, kCZ, kCY, kCX>, g, dim3(kNT), SR3<T, kCZ, kCY, kCX>::smem, s, f, f.phi2, c,
           zero_in ? 1 : 0);
  T* t = f.phi;
  f.phi = f.phi2;
  f.phi2 = t;
}

template <typename T>
void launch_prolong_smooth3d(Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  set_smem_attrs3<T>();
  dim3 g((unsigned)((f.mx - 1 + kTX - 1) / kTX), (unsigned)((f.my - 1 + kTY - 1) / kTY),
         (unsigned)((f.mz - 1 + kTZ - 1) / kTZ));
  launch_k(k_prolong_smooth3d<T, kTZ, kTY, kTX>, g, dim3(kNT), PS3<T, kTZ, kTY, kTX>::smem, s, f, f.phi2, c);
  T* t = f.phi;
  f.phi = f.phi2;
  f.phi2 = t;
}

void prepare_fused_ops3d() {
  set_smem_attrs3<float>();
  set_smem_attrs3<double>();
}

template void launch_smooth_restrict3d<float>(Lvl<float>&, const Lvl<float>&, bool, cudaStream_t);
template void launch_smooth_restrict3d<double>(Lvl<double>&, const Lvl<double>&, bool, cudaStream_t);
template void launch_prolong_smooth3d<float>(Lvl<float>&, const Lvl<float>&, cudaStream_t);
template void launch_prolong_smooth3d<double>(Lvl<double>&, const Lvl<double>&, cudaStream_t);

}  // namespace jmg
