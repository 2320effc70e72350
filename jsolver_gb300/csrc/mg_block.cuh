// mg_block.cuh — the multigrid operators run by one thread block over a whole level,
// with a block barrier after each pass, and the coarse recursion over them: the
// single-block coarse cycles (k_coarse_cycle over global memory, k_coarse_staged over
// shared memory) and the single-block coarse segments of the adjoint
// (mg_adjoint_kernels.cu) use them.
// Each pass evaluates the same per-point functions (mg_common.cuh) as the grid-wide
// kernels, so a level gives the same bits whichever runs it.
#pragma once

#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

template <typename T, int DIM>
__device__ void blk_sweep(const Lvl<T>& a) {
  const int nt = blockDim.x;
  for (int color = 0; color < 2; ++color) {
    if (DIM == 2) {
      const int hx = a.mx / 2;  // points of one colour per row (m even) -- m >= 2
      const int rows = a.my - 1;
      const int n = hx * rows;
      if (a.xll) {
        // 9-point stencil: the colour's two sub-lattices in the reference's order, rows
        // of parity 1 then 0 for red, 0 then 1 for black (solver_2d.py:684)
        for (int half = 0; half < 2; ++half) {
          const int rp = color == 0 ? 1 - half : half;
          for (int t = threadIdx.x; t < n; t += nt) {
            const int i = 2 + t / hx;
            if ((i & 1) != rp) continue;
            const int j = 2 + ((i + color) & 1) + 2 * (t % hx);
            if (j > a.mx) continue;
            const long long p = (long long)i * a.P + j;
            a.phi[p] = gs_point2d<T>(a, p);
          }
          if (half == 0) __syncthreads();
        }
      } else {
        for (int t = threadIdx.x; t < n; t += nt) {
          const int i = 2 + t / hx;
          const int j = 2 + ((i + color) & 1) + 2 * (t % hx);
          if (j > a.mx) continue;
          const long long p = (long long)i * a.P + j;
          a.phi[p] = gs_point2d<T>(a.phi, a.rhs, a.wx, a.wy, a.invd, p, a.P);
        }
      }
    } else {
      const int hx = a.mx / 2;
      const int ny = a.my - 1, nz = a.mz - 1;
      const int n = hx * ny * nz;
      const int par = (first_color_parity<3>() + color) & 1;
      for (int t = threadIdx.x; t < n; t += nt) {
        const int r = t / hx;
        const int j = 2 + r % ny, k = 2 + r / ny;
        const int i = 2 + ((j + k + par) & 1) + 2 * (t % hx);
        if (i > a.mx) continue;
        const long long p = (long long)k * a.S + (long long)j * a.P + i;
        a.phi[p] = gs_point3d<T>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.invd, p, a.P, a.S);
      }
    }
    __syncthreads();
  }
}

template <typename T, int DIM>
__device__ void blk_restrict(const Lvl<T>& f, const Lvl<T>& c) {
  const int nx = c.mx + 3, ny = c.my + 3, nz = DIM == 3 ? c.mz + 3 : 1;
  const int n = nx * ny * nz;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int I = t % nx, J = (t / nx) % ny, K = t / (nx * ny);
    const long long q = (long long)K * c.S + (long long)J * c.P + I;
    T v = T(0);
    if (DIM == 2) {
      if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) v = restrict_point2d<T>(f, J, I);
    } else {
      if (K >= 2 && K <= c.mz && J >= 2 && J <= c.my && I >= 2 && I <= c.mx) v = restrict_point3d<T>(f, K, J, I);
    }
    c.rhs[q] = v;
    c.phi[q] = T(0);
  }
  __syncthreads();
}

// by coarse cells (prolong_cell2d/3d): one thread updates the 4 (2D) or 8 (3D) fine
// points of a cell from its corners, without divergence between classes
template <typename T, int DIM>
__device__ void blk_prolong(const Lvl<T>& f, const Lvl<T>& c, bool diag) {
  const int nx = c.mx, ny = c.my, nz = DIM == 3 ? c.mz : 1;
  const int n = nx * ny * nz;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int I = 1 + t % nx, J = 1 + (t / nx) % ny, K = 1 + t / (nx * ny);
    if (DIM == 2) prolong_cell2d<T>(f, c, J, I, diag);
    else prolong_cell3d<T>(f, c, K, J, I, diag);
  }
  __syncthreads();
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
