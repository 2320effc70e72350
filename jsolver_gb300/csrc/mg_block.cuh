// mg_block.cuh — the multigrid operators run by one thread block over a whole level,
// with a block barrier after each pass, and the coarse recursion over them: the
// single-block coarse cycles (k_coarse_cycle over global memory, k_coarse_staged over
// shared memory) and the single-block coarse segments of the adjoint
// (mg_adjoint_kernels.cu) use them.
// Each pass evaluates the same per-point functions (mg_common.cuh) as the grid-wide
// kernels, so a level gives the same bits whichever runs it.
#pragma once

#include <cstdlib>

#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

// Level sizes are powers of two on every axis (the grid rule), so the passes map a thread
// index to a point with shifts and masks: an integer division by a run-time divisor per
// point was the largest part of a pass's latency on the small levels.
__device__ __forceinline__ int log2_pow2(int v) { return __ffs(v) - 1; }

template <typename T, int DIM>
__device__ void blk_sweep(const Lvl<T>& a) {
  const int nt = blockDim.x;
  for (int color = 0; color < 2; ++color) {
    if (DIM == 2) {
      const int hx = a.mx / 2;  // points of one colour per row (m even) -- m >= 2
      const int sh = log2_pow2(hx);
      const int rows = a.my - 1;
      const int n = hx * rows;
      if (a.xll) {
        // 9-point stencil: the colour's two sub-lattices in the reference's order, rows
        // of parity 1 then 0 for red, 0 then 1 for black (solver_2d.py:684)
        for (int half = 0; half < 2; ++half) {
          const int rp = color == 0 ? 1 - half : half;
          for (int t = threadIdx.x; t < n; t += nt) {
            const int i = 2 + (t >> sh);
            if ((i & 1) != rp) continue;
            const int j = 2 + ((i + color) & 1) + 2 * (t & (hx - 1));
            if (j > a.mx) continue;
            const long long p = (long long)i * a.P + j;
            a.phi[p] = gs_point2d<T>(a, p);
          }
          if (half == 0) __syncthreads();
        }
      } else {
        for (int t = threadIdx.x; t < n; t += nt) {
          const int i = 2 + (t >> sh);
          const int j = 2 + ((i + color) & 1) + 2 * (t & (hx - 1));
          if (j > a.mx) continue;
          const long long p = (long long)i * a.P + j;
          a.phi[p] = gs_point2d<T>(a.phi, a.rhs, a.wx, a.wy, a.invd, p, a.P);
        }
      }
    } else {
      // rows j run over 2 .. my + 1 (a power-of-two count), the last one skipped
      const int hx = a.mx / 2, shx = log2_pow2(hx), shy = log2_pow2(a.my);
      const int n = (hx * a.my) * (a.mz - 1);
      const int par = (first_color_parity<3>() + color) & 1;
      for (int t = threadIdx.x; t < n; t += nt) {
        const int r = t >> shx;
        const int j = 2 + (r & (a.my - 1)), k = 2 + (r >> shy);
        const int i = 2 + ((j + k + par) & 1) + 2 * (t & (hx - 1));
        if (j > a.my || i > a.mx) continue;
        const long long p = (long long)k * a.S + (long long)j * a.P + i;
        a.phi[p] = gs_point3d<T>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.invd, p, a.P, a.S);
      }
    }
    __syncthreads();
  }
}

// phi_c = 0 and rhs_c = 0 over the whole coarse array (one linear pass, no index
// arithmetic), then rhs_c = restricted defect at the interior points, enumerated with
// shifts over m_c per axis (the index m_c + 1 skipped)
template <typename T, int DIM>
__device__ void blk_restrict(const Lvl<T>& f, const Lvl<T>& c) {
  const long long e = DIM == 3 ? c.S * (long long)(c.mz + 3) : (long long)c.P * (c.my + 3);
  for (long long t = threadIdx.x; t < e; t += blockDim.x) {
    c.rhs[t] = T(0);
    c.phi[t] = T(0);
  }
  __syncthreads();
  const int shx = log2_pow2(c.mx), shy = log2_pow2(c.my);
  const int n = (c.mx * c.my) * (DIM == 3 ? c.mz : 1);
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int I = 2 + (t & (c.mx - 1)), J = 2 + ((t >> shx) & (c.my - 1)), K = 2 + (t >> (shx + shy));
    if (I > c.mx || J > c.my || (DIM == 3 && K > c.mz)) continue;
    if (DIM == 2) c.rhs[(long long)J * c.P + I] = restrict_point2d<T>(f, J, I);
    else c.rhs[(long long)K * c.S + (long long)J * c.P + I] = restrict_point3d<T>(f, K, J, I);
  }
  __syncthreads();
}

// by coarse cells (prolong_cell2d/3d): one thread updates the 4 (2D) or 8 (3D) fine
// points of a cell from its corners, without divergence between classes
template <typename T, int DIM>
__device__ void blk_prolong(const Lvl<T>& f, const Lvl<T>& c, bool diag) {
  const int nx = c.mx, ny = c.my, nz = DIM == 3 ? c.mz : 1;
  const int n = nx * ny * nz, shx = log2_pow2(nx), shy = log2_pow2(ny);
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int I = 1 + (t & (nx - 1)), J = 1 + ((t >> shx) & (ny - 1)), K = 1 + (t >> (shx + shy));
    if (DIM == 2) prolong_cell2d<T>(f, c, J, I, diag);
    else prolong_cell3d<T>(f, c, K, J, I, diag);
  }
  __syncthreads();
}

// The coarse sub-cycle as a list of operations, built on the host in the order of the
// recursion below (solver_2d.py:582-614): one byte per operation, (kind << 5) | level.
// Walking the list costs a shared-memory byte read per operation instead of the frame
// stack's local-memory bookkeeping. n = 0: no list (the schedule did not fit), the
// kernel walks the recursion itself.
constexpr int kMaxCoarseOps = 1000;
enum { kCoarseSweep = 0, kCoarseRestrict = 1, kCoarseProlong = 2 };
struct CoarseOps {
  int n;
  unsigned char op[kMaxCoarseOps];
};

// copy of the list into shared memory (before the kernel's first barrier)
__device__ __forceinline__ void stage_coarse_ops(const CoarseOps& src, CoarseOps* dst) {
  if (threadIdx.x == 0) dst->n = src.n;
  for (int k = threadIdx.x; k < src.n; k += blockDim.x) dst->op[k] = src.op[k];
}

template <typename T, int DIM>
__device__ void blk_run(const LvlTable<T>* __restrict__ tab, const CycleParams& cp, const CoarseOps* ops) {
  const int n = ops->n;
  for (int o = 0; o < n; ++o) {
    const int op = ops->op[o], lev = op & 31;
    const Lvl<T>& a = tab->l[lev];
    if ((op >> 5) == kCoarseSweep) blk_sweep<T, DIM>(a);
    else if ((op >> 5) == kCoarseRestrict) blk_restrict<T, DIM>(a, tab->l[lev + 1]);
    else blk_prolong<T, DIM>(a, tab->l[lev + 1], cp.diag != 0);
  }
}

// host: the list of the sub-cycle from lev0 (the same schedule as blk_cycle); n = 0 when
// it exceeds kMaxCoarseOps
inline void coarse_ops_rec(const CycleParams& cp, int lev, bool fcycle, bool skip_pre, CoarseOps& o) {
  auto push = [&](int kind, int l) {
    if (o.n >= 0 && o.n < kMaxCoarseOps) o.op[o.n++] = (unsigned char)((kind << 5) | l);
    else o.n = -1;
  };
  if (lev == cp.last_level) {
    for (int k = 0; k < cp.nu1 + cp.nu2; ++k) push(kCoarseSweep, lev);
    return;
  }
  if (!skip_pre)
    for (int k = 0; k < cp.nu1; ++k) push(kCoarseSweep, lev);
  push(kCoarseRestrict, lev);
  if (fcycle)
    for (int g = 0; g < cp.gamma; ++g) coarse_ops_rec(cp, lev + 1, true, false, o);
  for (int g = 0; g < cp.gamma; ++g) coarse_ops_rec(cp, lev + 1, false, false, o);
  push(kCoarseProlong, lev);
  for (int k = 0; k < cp.nu2; ++k) push(kCoarseSweep, lev);
}

inline CoarseOps coarse_ops(const CycleParams& cp, int lev0, bool fcycle, bool skip_pre) {
  CoarseOps o;
  o.n = 0;
  const char* e = getenv("JMG_COARSE_OPS");  // "0": walk the recursion (the checker of the list)
  if (cp.last_level < 32 && !(e && e[0] == '0')) coarse_ops_rec(cp, lev0, fcycle, skip_pre, o);
  if (o.n < 0) o.n = 0;
  return o;
}

// multigrid_cycle (solver_2d.py:582-614) restricted to levels >= lev, run by one block.
// The recursion is unrolled into an explicit stack of frames (no device recursion, so the
// per-thread stack stays within its default size). Every thread walks the same frames,
// so the __syncthreads inside the operators are reached uniformly.
template <typename T, int DIM>
__device__ void blk_cycle(const LvlTable<T>* __restrict__ tab, const CycleParams& cp, int lev0, bool fcycle0,
                          bool skip_pre0) {
  struct Frame {
    int lev, stage, g;
    bool fcycle, skip_pre;
  };
  Frame st[kMaxLevels + 1];
  int sp = 0;
  st[sp++] = Frame{lev0, 0, 0, fcycle0, skip_pre0};
  while (sp > 0) {
    Frame& f = st[sp - 1];
    const Lvl<T> a = tab->l[f.lev];
    if (f.lev == cp.last_level) {
      for (int s = 0; s < cp.nu1 + cp.nu2; ++s) blk_sweep<T, DIM>(a);
      --sp;
      continue;
    }
    if (f.stage == 0) {
      if (!f.skip_pre)
        for (int s = 0; s < cp.nu1; ++s) blk_sweep<T, DIM>(a);
      blk_restrict<T, DIM>(a, tab->l[f.lev + 1]);
      f.stage = f.fcycle ? 1 : 2;
      f.g = 0;
    }
    if (f.stage == 1) {  // F-cycle: gamma recursive F-cycles first (solver_2d.py:609-610)
      if (f.g < cp.gamma) {
        ++f.g;
        st[sp++] = Frame{f.lev + 1, 0, 0, true, false};
        continue;
      }
      f.stage = 2;
      f.g = 0;
    }
    if (f.stage == 2) {  // gamma plain cycles (solver_2d.py:611)
      if (f.g < cp.gamma) {
        ++f.g;
        st[sp++] = Frame{f.lev + 1, 0, 0, false, false};
        continue;
      }
      f.stage = 3;
    }
    blk_prolong<T, DIM>(a, tab->l[f.lev + 1], cp.diag != 0);
    for (int s = 0; s < cp.nu2; ++s) blk_sweep<T, DIM>(a);
    --sp;
  }
}

}  // namespace jmg
