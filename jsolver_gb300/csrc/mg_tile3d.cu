// mg_tile3d.cu — 3D defect + restriction with every fine defect computed once, and the
// 3D prolongation by coarse cells.
//
// The coarse right-hand side at (K, J, I) is 1/32 of the defects at the 12 red fine
// points around (2K-1, 2J-1, 2I-1) that differ from it in two coordinates by 1, plus 1/8
// of the defect at that centre (solver_3d.py:622-652). One thread per coarse point (the
// grid-wide k_restrict3d) evaluates 13 defects: about three times the red defects of the
// level, each one's loads waiting behind the last. Here a block takes a tile of
// CK x CJ x CI coarse points: it stages the fine phi of the tile's footprint (with a
// one-point halo) in shared memory, computes each red defect of the footprint once into
// shared memory, then forms every coarse value. The defect and the sum are evaluated in
// the order of defect_point3d and restrict_point3d, so the result is bit-identical to
// k_restrict3d. Also phi_c = 0 on the whole padded coarse box.
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_dual.cuh"

namespace jmg {

namespace {

template <typename T, int CK, int CJ, int CI>
__global__ void __launch_bounds__(CK * CJ * CI) k_restrict_tile3d(Lvl<T> f, Lvl<T> c) {
  pdl_enter();
  constexpr int DK = 2 * CK + 1, DJ = 2 * CJ + 1, DI = 2 * CI + 1;  // defect footprint
  constexpr int FK = DK + 2, FJ = DJ + 2, FI = DI + 2;              // with the halo
  constexpr int NT = CK * CJ * CI;
  constexpr int NPHI = FK * FJ * FI;
  constexpr int XR = (DI + 1) / 2;  // red candidates per footprint row
  constexpr int NRED = DK * DJ * XR;
  __shared__ T Phi[FK][FJ][FI];
  __shared__ T Def[DK][DJ][DI];
  const int K0 = blockIdx.z * CK, J0 = blockIdx.y * CJ, I0 = blockIdx.x * CI;
  const int dk0 = 2 * K0 - 2, dj0 = 2 * J0 - 2, di0 = 2 * I0 - 2;  // fine index of Def[0][0][0]
  const int tid = threadIdx.x;
  const int P = f.P;
  const long long S = f.S;
  // 1. fine phi of the footprint and its halo (zero outside the padded array). Every
  //    thread issues all its loads before the first store, in batches of eight.
  constexpr int U1 = (NPHI + NT - 1) / NT;
#pragma unroll
  for (int h = 0; h < U1; h += 8) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = tid + (h + u) * NT;
      v[u] = T(0);
      if (h + u < U1 && t < NPHI) {
        const int a = t / (FJ * FI), rem = t - a * (FJ * FI);
        const int b = rem / FI, q = rem - b * FI;
        const int k = dk0 - 1 + a, j = dj0 - 1 + b, i = di0 - 1 + q;
        if (k >= 0 && j >= 0 && i >= 0 && k <= f.mz + 2 && j <= f.my + 2 && i <= f.mx + 2)
          v[u] = f.phi[(long long)k * S + (long long)j * P + i];
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = tid + (h + u) * NT;
      if (h + u < U1 && t < NPHI) (&Phi[0][0][0])[t] = v[u];
    }
  }
  __syncthreads();
  // 2. defects at the red fine points of the footprint (i + j + k odd) that are interior;
  //    the coarse values below read only those. Three points per batch, loads first.
  constexpr int U2 = (NRED + NT - 1) / NT;
#pragma unroll
  for (int h = 0; h < U2; h += 3) {
    T ac[3], wxm[3], wxp[3], wym[3], wyp[3], wzm[3], wzp[3], rh[3];
    int pos[3];
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int t = tid + (h + u) * NT;
      pos[u] = -1;
      if (h + u < U2 && t < NRED) {
        const int a = t / (DJ * XR), rem = t - a * (DJ * XR);
        const int b = rem / XR, xp = rem - b * XR;
        const int k = dk0 + a, j = dj0 + b;
        const int q = 2 * xp + ((1 - k - j - di0) & 1);  // i = di0 + q has i + j + k odd
        const int i = di0 + q;
        if (q < DI && k >= 2 && k <= f.mz && j >= 2 && j <= f.my && i >= 2 && i <= f.mx) {
          const long long p = (long long)k * S + (long long)j * P + i;
          pos[u] = (a * DJ + b) * DI + q;
          ac[u] = f.acc[p];
          wxm[u] = f.wx[p - 1];
          wxp[u] = f.wx[p];
          wym[u] = f.wy[p - P];
          wyp[u] = f.wy[p];
          wzm[u] = f.wz[p - S];
          wzp[u] = f.wz[p];
          rh[u] = f.rhs[p];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      if (pos[u] < 0) continue;
      const int a = pos[u] / (DJ * DI), rem = pos[u] - a * (DJ * DI);
      const int b = rem / DI, q = rem - b * DI;
      const int aa = a + 1, bb = b + 1, qq = q + 1;  // position in Phi
      // defect_point3d's order
      T d = ac[u] * Phi[aa][bb][qq];
      d = fma(-wxm[u], Phi[aa][bb][qq - 1], d);
      d = fma(-wxp[u], Phi[aa][bb][qq + 1], d);
      d = fma(-wym[u], Phi[aa][bb - 1][qq], d);
      d = fma(-wyp[u], Phi[aa][bb + 1][qq], d);
      d = fma(-wzm[u], Phi[aa - 1][bb][qq], d);
      d = fma(-wzp[u], Phi[aa + 1][bb][qq], d);
      Def[a][b][q] = d + rh[u];
    }
  }
  __syncthreads();
  // 3. one coarse point per thread, over the whole padded coarse box
  {
    const int a = tid / (CJ * CI), rem = tid - a * (CJ * CI);
    const int b = rem / CI, q = rem - b * CI;
    const int K = K0 + a, J = J0 + b, I = I0 + q;
    if (K <= c.mz + 2 && J <= c.my + 2 && I <= c.mx + 2) {
      T v = T(0);
      if (K >= 2 && K <= c.mz && J >= 2 && J <= c.my && I >= 2 && I <= c.mx) {
        const int x = 2 * K - 1 - dk0, y = 2 * J - 1 - dj0, z = 2 * I - 1 - di0;  // centre in Def
        // restrict_point3d's order: (+P+1), (+P-1), (-P+1), (-P-1), (+S+1), (+S-1),
        // (-S+1), (-S-1), (+S+P), (+S-P), (-S+P), (-S-P), then the centre
        T s = Def[x][y + 1][z + 1];
        s = s + Def[x][y + 1][z - 1];
        s = s + Def[x][y - 1][z + 1];
        s = s + Def[x][y - 1][z - 1];
        s = s + Def[x + 1][y][z + 1];
        s = s + Def[x + 1][y][z - 1];
        s = s + Def[x - 1][y][z + 1];
        s = s + Def[x - 1][y][z - 1];
        s = s + Def[x + 1][y + 1][z];
        s = s + Def[x + 1][y - 1][z];
        s = s + Def[x - 1][y + 1][z];
        s = s + Def[x - 1][y - 1][z];
        v = T(0.03125) * s + T(0.125) * Def[x][y][z];
      }
      const long long qc = (long long)K * c.S + (long long)J * c.P + I;
      c.rhs[qc] = v;
      c.phi[qc] = T(0);
    }
  }
}

// ---- prolongation --------------------------------------------------------------------
// phi_f += P phi_c (solver_3d.py:654-677) by coarse cells: a thread takes the 2 x 2 x 2
// fine points (2K-1 .. 2K, 2J-1 .. 2J, 2I-1 .. 2I), which all interpolate from the eight
// coarse corners (K .. K+1, J .. J+1, I .. I+1). It loads those once and forms each fine
// value with prolong_point3d's formula for its class (odd/even indices), in the same
// order, so the result is bit-identical to k_prolong3d; points with exactly two even
// indices are skipped unless bilinear (nu2 <= 0), as there. One thread per fine point
// spent ~80 instructions per point on 64-bit index arithmetic and branches that diverge
// between neighbouring points; here the arithmetic is shared by eight points.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong3d_cells(Lvl<T> f, Lvl<T> c, int bilinear) {
  pdl_enter();
  const int I = 1 + blockIdx.x * blockDim.x + threadIdx.x;  // cells 1 .. m_c per axis
  const int J = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int K = 1 + blockIdx.z;
  if (I > c.mx || J > c.my) return;
  prolong_cell3d<T>(f, c, K, J, I, bilinear != 0);
}

// Tiles: FP32 4 x 4 x 16 coarse points (256 threads, 27.6 KB of shared memory), FP64
// 4 x 4 x 8 (128 threads, 29.4 KB).
template <typename T>
struct Tile3;
template <>
struct Tile3<float> {
  static constexpr int CK = 4, CJ = 4, CI = 16;
};
template <>
struct Tile3<double> {
  static constexpr int CK = 4, CJ = 4, CI = 8;
};

}  // namespace

template <typename T>
void launch_restrict_tile3d(const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  constexpr int CK = Tile3<T>::CK, CJ = Tile3<T>::CJ, CI = Tile3<T>::CI;
  dim3 g((unsigned)((c.mx + 3 + CI - 1) / CI), (unsigned)((c.my + 3 + CJ - 1) / CJ),
         (unsigned)((c.mz + 3 + CK - 1) / CK));
  launch_k(k_restrict_tile3d<T, CK, CJ, CI>, g, dim3(CK * CJ * CI), 0, s, f, c);
}

template <typename T>
void launch_prolong_cells3d(const Lvl<T>& f, const Lvl<T>& c, int bilinear, cudaStream_t s) {
  dim3 b(32, 8, 1), g((unsigned)((c.mx + 31) / 32), (unsigned)((c.my + 7) / 8), (unsigned)c.mz);
  launch_k(k_prolong3d_cells<T>, g, b, 0, s, f, c, bilinear);
}

template void launch_prolong_cells3d<double>(const Lvl<double>&, const Lvl<double>&, int, cudaStream_t);
template void launch_prolong_cells3d<float>(const Lvl<float>&, const Lvl<float>&, int, cudaStream_t);
// the forward-mode solve (mg_tangent.cu)
template void launch_prolong_cells3d<Dual>(const Lvl<Dual>&, const Lvl<Dual>&, int, cudaStream_t);
template void launch_restrict_tile3d<double>(const Lvl<double>&, const Lvl<double>&, cudaStream_t);
template void launch_restrict_tile3d<float>(const Lvl<float>&, const Lvl<float>&, cudaStream_t);

}  // namespace jmg
