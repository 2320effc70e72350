// mg_fused.cu — one-pass red-black sweeps (both colours in one launch), 3D and 2D.
//
// The two colour passes of launch_sweep each stream every array of the level: the
// colours interleave within every cache line, so a pass that updates half the points
// still reads all of phi, rhs, the three face couplings and 1/A_cc. This kernel reads
// them once per sweep. Each block owns a tile of 64 x 8 interior columns (x, y) and a
// chunk of z-planes, and marches up the chunk keeping the new red values of four planes
// in shared memory. One step of the march, for plane k:
//   load the inputs of red(k+2) (the tile and a ring of one point around it, from the
//   old black values) into registers,
//   black(k) on the tile from the new red values of planes k-1, k, k+1, and write both
//   colours of plane k,
//   finish red(k+2) into shared memory, one barrier.
// The red loads go to DRAM; issuing them before the black update lets that update's
// loads (mostly L2 hits) run under their latency, and one barrier per plane suffices.
// Neighbouring tiles and chunks recompute the red values of their shared ring and
// boundary planes, so blocks never read what another block writes: the sweep reads phi
// and writes a second buffer (the level's phi2), and the caller swaps the two.
// Every value is computed with the arithmetic of gs_point3d in the same order, so the
// result is bit-identical to the two colour passes (solver_3d.py:679-706).
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

constexpr int kTX = 64;                      // interior points per tile row (32 threads x 2)
constexpr int kTY = 8;                       // interior rows per tile
constexpr int kRX = kTX + 2;                 // red ring: x from i0-1 to i0+64
constexpr int kRY = kTY + 2;                 // y from j0-1 to j0+8
constexpr int kRed = kRX * kRY / 2;          // red points of the ring region per plane (330)
constexpr int kThreads = 384;                // one red point per thread and plane
constexpr int kSlots = 4;                    // red planes k-1 .. k+2 live in one step
// Four blocks per SM (40 registers). FP64 levels sweep in one pass only on request
// (JMG_FUSED64=1): at four blocks per SM the FP64 form spills (375 us per 256^3 sweep),
// at two it does not but hides less latency (451 us); the colour passes take 287 us.
constexpr int kBlocksPerSM = 4;
template <typename T>
constexpr int kBlocksPerSMT = kBlocksPerSM;

// Inputs of one red value, loaded ahead of their use so that their DRAM latency overlaps
// the black update of an earlier plane; then the value, with gs_point3d's arithmetic.
// Offsets are 32-bit (levels of fewer than 2^31 points).
template <typename T>
struct RedIn {
  T wzp, pzp, wzm, pzm, wyp, pyp, wym, pym, wxp, pxp, wxm, pxm, rhs, invd;
};

template <typename T>
__device__ __forceinline__ void red_load(const Lvl<T>& a, int p, int P, int S, bool zero_in, RedIn<T>& r) {
  r.rhs = __ldg(a.rhs + p);
  r.invd = __ldg(a.invd + p);
  if (zero_in) return;
  r.wzp = __ldg(a.wz + p), r.pzp = __ldg(a.phi + p + S);
  r.wzm = __ldg(a.wz + p - S), r.pzm = __ldg(a.phi + p - S);
  r.wyp = __ldg(a.wy + p), r.pyp = __ldg(a.phi + p + P);
  r.wym = __ldg(a.wy + p - P), r.pym = __ldg(a.phi + p - P);
  r.wxp = __ldg(a.wx + p), r.pxp = __ldg(a.phi + p + 1);
  r.wxm = __ldg(a.wx + p - 1), r.pxm = __ldg(a.phi + p - 1);
}

template <typename T>
__device__ __forceinline__ T red_eval(const RedIn<T>& r, bool zero_in) {
  if (zero_in) return (T(0) - r.rhs) * r.invd;
  T s = r.wzp * r.pzp;
  s = fma(r.wzm, r.pzm, s);
  s = fma(r.wyp, r.pyp, s);
  s = fma(r.wym, r.pym, s);
  s = fma(r.wxp, r.pxp, s);
  s = fma(r.wxm, r.pxm, s);
  s = s - r.rhs;
  return s * r.invd;
}

template <typename T>
__global__ void __launch_bounds__(kThreads, kBlocksPerSMT<T>)
    k_sweep_fused3d(Lvl<T> a, T* __restrict__ out, int zero_in, int kchunk) {
  pdl_enter();
  __shared__ T red[kSlots][kRY][kRX];
  const int i0 = 2 + kTX * blockIdx.x;
  const int j0 = 2 + kTY * blockIdx.y;
  const int k0 = 2 + kchunk * blockIdx.z;
  const int k1 = min(k0 + kchunk, a.mz + 1);
  const bool zin = zero_in != 0;
  const int P = a.P, S = (int)a.S;
  const int par = first_color_parity<3>();
  const int t = threadIdx.x;
  // red role (t < kRed): one point of the ring region per plane, row rr, columns rx or
  // rx + 1 (the red one alternates with the plane's parity)
  const int rr = t / (kRX / 2);
  const int rx = 2 * (t - rr * (kRX / 2));  // column in the slot, 0 .. 64
  const int rj = j0 - 1 + rr;
  const bool red_role = t < kRed;
  const bool red_row_in = rj >= 2 && rj <= a.my;
  const int rpar = (par - rj - (i0 - 1) - rx) & 1;  // parity offset at plane 0
  const int rrow = rj * P + (i0 - 1) + rx;         // offset of column rx in plane 0
  // the red value of plane k: 0 outside the interior (the frame stays zero)
  auto red_at = [&](int k, int* slot_x) -> bool {
    const int off = (rpar - k) & 1;
    *slot_x = rx + off;
    const int i = i0 - 1 + rx + off;
    return red_row_in && i >= 2 && i <= a.mx && k >= 2 && k <= a.mz;
  };
  // prologue: red values of planes k0-1, k0, k0+1
  if (red_role) {
    for (int k = k0 - 1; k <= k0 + 1; ++k) {
      int x;
      T v = T(0);
      if (red_at(k, &x)) {
        RedIn<T> in;
        red_load<T>(a, k * S + rrow + (x - rx), P, S, zin, in);
        v = red_eval<T>(in, zin);
      }
      red[k & (kSlots - 1)][rr][x] = v;
    }
  }
  __syncthreads();
  // black role (t < 256): row j, the pair of columns ie, ie + 1
  const int tx = t & 31, ty = t >> 5;
  const int j = j0 + ty;
  const int ie = i0 + 2 * tx;
  const bool blk_role = ty < kTY && j <= a.my;
  const int bpar = (par - j - ie) & 1;
  const int brow = j * P + ie;
  const int lr = ty + 1;
  for (int k = k0; k < k1; ++k) {
    // 1. inputs of red(k+2), needed from the next step on (black(k+1) reads it)
    int x2 = 0;
    const bool next = red_role && k + 2 <= k1;
    const bool load2 = next && red_at(k + 2, &x2);
    RedIn<T> in;
    if (load2) red_load<T>(a, (k + 2) * S + rrow + (x2 - rx), P, S, zin, in);
    // 2. black(k) from the red values of planes k-1, k, k+1; both colours of plane k out
    if (blk_role) {
      const T(*rm)[kRX] = red[(k - 1) & (kSlots - 1)];
      const T(*rc)[kRX] = red[k & (kSlots - 1)];
      const T(*rp)[kRX] = red[(k + 1) & (kSlots - 1)];
      const int roff = (bpar - k) & 1;  // red one of the pair: ie + roff
      const int pr = k * S + brow + roff;
      const int pb = k * S + brow + (roff ^ 1);
      const int xr = ie + roff - (i0 - 1), xb = ie + (roff ^ 1) - (i0 - 1);
      if (ie + roff <= a.mx) out[pr] = rc[lr][xr];
      if (ie + (roff ^ 1) <= a.mx) {
        T s = __ldg(a.wz + pb) * rp[lr][xb];
        s = fma(__ldg(a.wz + pb - S), rm[lr][xb], s);
        s = fma(__ldg(a.wy + pb), rc[lr + 1][xb], s);
        s = fma(__ldg(a.wy + pb - P), rc[lr - 1][xb], s);
        s = fma(__ldg(a.wx + pb), rc[lr][xb + 1], s);
        s = fma(__ldg(a.wx + pb - 1), rc[lr][xb - 1], s);
        s = s - __ldg(a.rhs + pb);
        out[pb] = s * __ldg(a.invd + pb);
      }
    }
    // 3. red(k+2) into the slot black(k-1) read last step
    if (next) red[(k + 2) & (kSlots - 1)][rr][x2] = load2 ? red_eval<T>(in, zin) : T(0);
    __syncthreads();
  }
}

}  // namespace

// Planes per block. The grid is one wave (kBlocksPerSM resident blocks on each of 152
// SMs): a partial second wave would run at a fraction of the occupancy for a whole
// block's time. Chunks have at least 16 planes, so the three planes each chunk starts
// with stay a small share.
int fused_chunk3d(int mx, int my, int mz, int blocks_per_sm) {
  const long long tiles = (long long)((mx - 1 + kTX - 1) / kTX) * ((my - 1 + kTY - 1) / kTY);
  const long long resident = 152LL * blocks_per_sm;
  const int planes = mz - 1;
  long long nchunk = resident / tiles;
  const long long maxchunk = (planes + 15) / 16;
  if (nchunk > maxchunk) nchunk = maxchunk;
  if (nchunk < 1) nchunk = 1;
  return (int)((planes + nchunk - 1) / nchunk);
}

int fused_blocks3d(int mx, int my, int mz) {
  const int kchunk = fused_chunk3d(mx, my, mz, kBlocksPerSM);
  return ((mx - 1 + kTX - 1) / kTX) * ((my - 1 + kTY - 1) / kTY) * ((mz - 1 + kchunk - 1) / kchunk);
}

// the share of one full wave the one-pass grid fills, in thousandths
int fused_wave_permille(int mx, int my, int mz) {
  return (int)(1000LL * fused_blocks3d(mx, my, mz) / (152LL * kBlocksPerSM));
}

template <typename T>
void launch_sweep_fused3d(Lvl<T>& a, bool zero_in, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (sweep_tma3d_enabled() && launch_sweep_tma3d(a, zero_in, s)) return;
  }
  const int kchunk = fused_chunk3d(a.mx, a.my, a.mz, kBlocksPerSMT<T>);
  dim3 g((a.mx - 1 + kTX - 1) / kTX, (a.my - 1 + kTY - 1) / kTY, (a.mz - 1 + kchunk - 1) / kchunk);
  launch_k(k_sweep_fused3d<T>, g, dim3(kThreads), 0, s, a, a.phi2, zero_in ? 1 : 0, kchunk);
  T* t = a.phi;
  a.phi = a.phi2;
  a.phi2 = t;
}

// ---- 2D -------------------------------------------------------------------------------
// A 2D level of 1024^2 stays in L2 during a solve, so a march in y would wait on every
// row; one block instead takes a 64 x 16 tile whole: the old phi of the tile with a
// two-point halo into shared memory, the red values of the tile and a one-point ring from
// it, one barrier, then the black values of the tile. Each phase's global loads are
// issued before their first use. Same bits as the colour passes (gs_point2d's order).
namespace {

constexpr int k2TX = 64, k2TY = 16;
constexpr int k2PX = k2TX + 4, k2PY = k2TY + 4;  // old phi, x from i0-2, y from j0-2
constexpr int k2RX = k2TX + 2, k2RY = k2TY + 2;  // red ring, x from i0-1, y from j0-1
constexpr int k2Threads = 256;
constexpr int k2Red = k2RX * k2RY / 2;           // 594 red points in the ring region
constexpr int k2Blk = k2TX * k2TY / 2;           // 512 black points in the tile

template <typename T>
__global__ void __launch_bounds__(k2Threads) k_sweep_onepass2d(Lvl<T> a, T* __restrict__ out, int zero_in) {
  pdl_enter();
  __shared__ T Ph[k2PY][k2PX];
  __shared__ T Rd[k2RY][k2RX];
  const int i0 = 2 + k2TX * blockIdx.x, j0 = 2 + k2TY * blockIdx.y;
  const int tid = threadIdx.x;
  const int P = a.P;
  const bool zin = zero_in != 0;
  // 1. old phi with a two-point halo (zero outside the padded array; unused with zero_in)
  constexpr int NPH = k2PX * k2PY, U1 = (NPH + k2Threads - 1) / k2Threads;
  if (!zin) {
    T v[U1];
#pragma unroll
    for (int u = 0; u < U1; ++u) {
      const int t = tid + u * k2Threads;
      v[u] = T(0);
      if (t < NPH) {
        const int r = t / k2PX, q = t - r * k2PX;
        const int j = j0 - 2 + r, i = i0 - 2 + q;
        if (j >= 0 && i >= 0 && j <= a.my + 2 && i <= a.mx + 2) v[u] = a.phi[(long long)j * P + i];
      }
    }
#pragma unroll
    for (int u = 0; u < U1; ++u) {
      const int t = tid + u * k2Threads;
      if (t < NPH) (&Ph[0][0])[t] = v[u];
    }
  }
  // coefficients of the thread's red points (ring region, i + j even)
  constexpr int U2 = (k2Red + k2Threads - 1) / k2Threads;
  T rwxm[U2], rwxp[U2], rwym[U2], rwyp[U2], rrh[U2], rinv[U2];
  int rpos[U2];  // r * k2RX + x in the red slots, -1 where the point is not interior
#pragma unroll
  for (int u = 0; u < U2; ++u) {
    const int t = tid + u * k2Threads;
    rpos[u] = -2;  // -2: no point; -1: a ring point outside the interior (value 0)
    if (t < k2Red) {
      const int r = t / (k2RX / 2), xp = t - r * (k2RX / 2);
      const int j = j0 - 1 + r;
      const int x = 2 * xp + ((j + i0 - 1) & 1);  // i = i0 - 1 + x with i + j even
      const int i = i0 - 1 + x;
      rpos[u] = -(r * k2RX + x) - 3;  // encoded slot of an exterior point
      if (j >= 2 && j <= a.my && i >= 2 && i <= a.mx) {
        const long long p = (long long)j * P + i;
        rpos[u] = r * k2RX + x;
        rrh[u] = a.rhs[p];
        rinv[u] = a.invd[p];
        if (!zin) {
          rwxm[u] = a.wx[p - 1];
          rwxp[u] = a.wx[p];
          rwym[u] = a.wy[p - P];
          rwyp[u] = a.wy[p];
        }
      }
    }
  }
  __syncthreads();
  // coefficients of the thread's black points of the tile, issued before the red values
  constexpr int U3 = k2Blk / k2Threads;  // 2
  T bwxm[U3], bwxp[U3], bwym[U3], bwyp[U3], brh[U3], binv[U3];
  long long bp[U3];
  int bj[U3], bi[U3];
#pragma unroll
  for (int u = 0; u < U3; ++u) {
    const int t = tid + u * k2Threads;
    const int r = t / (k2TX / 2), xp = t - r * (k2TX / 2);
    const int j = j0 + r;
    const int i = i0 + 2 * xp + ((j + i0 + 1) & 1);  // i + j odd
    bj[u] = j;
    bi[u] = i;
    bp[u] = (long long)j * P + i;
    if (j <= a.my && i <= a.mx) {
      const long long p = bp[u];
      bwxm[u] = a.wx[p - 1];
      bwxp[u] = a.wx[p];
      bwym[u] = a.wy[p - P];
      bwyp[u] = a.wy[p];
      brh[u] = a.rhs[p];
      binv[u] = a.invd[p];
    }
  }
  // 2. red values of the ring region (gs_point2d's order)
#pragma unroll
  for (int u = 0; u < U2; ++u) {
    if (rpos[u] == -2) continue;
    if (rpos[u] < 0) {  // exterior ring point: the frame stays zero
      (&Rd[0][0])[-(rpos[u] + 3)] = T(0);
      continue;
    }
    const int r = rpos[u] / k2RX, x = rpos[u] - r * k2RX;
    T v;
    if (zin) {
      v = (T(0) - rrh[u]) * rinv[u];
    } else {
      const int pr = r + 1, px = x + 1;  // position in Ph
      T s = rwyp[u] * Ph[pr + 1][px];
      s = fma(rwym[u], Ph[pr - 1][px], s);
      s = fma(rwxp[u], Ph[pr][px + 1], s);
      s = fma(rwxm[u], Ph[pr][px - 1], s);
      s = s - rrh[u];
      v = s * rinv[u];
    }
    Rd[r][x] = v;
  }
  __syncthreads();
  // 3. black values of the tile from the new red values; both colours of the tile out
#pragma unroll
  for (int u = 0; u < U3; ++u) {
    const int j = bj[u], i = bi[u];
    if (j > a.my) continue;
    const int r = j - (j0 - 1), x = i - (i0 - 1);  // position in Rd
    if (i <= a.mx) {
      T s = bwyp[u] * Rd[r + 1][x];
      s = fma(bwym[u], Rd[r - 1][x], s);
      s = fma(bwxp[u], Rd[r][x + 1], s);
      s = fma(bwxm[u], Rd[r][x - 1], s);
      s = s - brh[u];
      out[bp[u]] = s * binv[u];
    }
  }
  // red values of the tile
  for (int t = tid; t < k2Blk; t += k2Threads) {
    const int r = t / (k2TX / 2), xp = t - r * (k2TX / 2);
    const int j = j0 + r;
    const int i = i0 + 2 * xp + ((j + i0) & 1);  // i + j even
    if (j <= a.my && i <= a.mx) out[(long long)j * P + i] = Rd[j - (j0 - 1)][i - (i0 - 1)];
  }
}

}  // namespace

template <typename T>
void launch_sweep_onepass2d(Lvl<T>& a, bool zero_in, cudaStream_t s) {
  dim3 g((a.mx - 1 + k2TX - 1) / k2TX, (a.my - 1 + k2TY - 1) / k2TY);
  launch_k(k_sweep_onepass2d<T>, g, dim3(k2Threads), 0, s, a, a.phi2, zero_in ? 1 : 0);
  T* t = a.phi;
  a.phi = a.phi2;
  a.phi2 = t;
}

template void launch_sweep_onepass2d<double>(Lvl<double>&, bool, cudaStream_t);
template void launch_sweep_onepass2d<float>(Lvl<float>&, bool, cudaStream_t);

template void launch_sweep_fused3d<double>(Lvl<double>&, bool, cudaStream_t);
template void launch_sweep_fused3d<float>(Lvl<float>&, bool, cudaStream_t);

}  // namespace jmg

namespace jmg {

template <typename T>
void launch_sweep_onepass(int dim, Lvl<T>& a, bool zero_in, cudaStream_t s) {
  if (dim == 3) launch_sweep_fused3d<T>(a, zero_in, s);
  else launch_sweep_onepass2d<T>(a, zero_in, s);
}

template void launch_sweep_onepass<double>(int, Lvl<double>&, bool, cudaStream_t);
template void launch_sweep_onepass<float>(int, Lvl<float>&, bool, cudaStream_t);

}  // namespace jmg
