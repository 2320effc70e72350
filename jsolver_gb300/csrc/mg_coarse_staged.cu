// mg_coarse_staged.cu — the coarse sub-cycle on one thread block, with every array of the
// coarse levels in shared memory, staged by the bulk-copy engine.
//
// The coarse levels (a few thousand points) are bound by the latency of the recursion's
// dependent passes (solver_2d.py:582-614: two sweeps, a restriction and a prolongation per
// level, about 28 passes from 2D 32^2 down), so every pass should read shared memory, not
// L2, and the staging must not add round trips of its own. One thread issues all copies
// at once as cp.async.bulk transfers into shared memory, completing on one mbarrier:
//   * the coefficients of every coarse level (face couplings, 1/A_cc, A_cc, and the D_xy
//     diagonals where present) before the programmatic-launch wait, since the cycle never
//     writes them, so their transfer overlaps the end of the preceding kernel;
//   * phi and rhs of the first coarse level after it (the preceding restriction wrote them).
// The deeper levels' phi and rhs are produced in shared memory by the recursion itself
// (each restriction writes rhs_c and zeroes phi_c). The arrays keep the workspace's
// pitched layout, so one copy moves a whole array and the level views differ from the
// global ones only in their pointers. The passes are the single-block operators of
// mg_block.cuh (the same per-point functions as every other path), so the results are the
// bits of k_coarse_cycle. At the end phi of the first coarse level goes back to global
// memory; the deeper levels are private to the launch.
//
// The wait on the mbarrier is bounded: if the transfer has not completed after a fixed
// number of polls, the block raises the table's fault flag, fills phi of the first coarse
// level with NaN (so that the solve's result shows the failure), waits again (bounded) for
// its copies in flight and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "mg_block.cuh"
#include "mg_bulk.cuh"
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

template <typename T, int DIM>
__host__ __device__ inline int staged_arrays(bool offdiag) {
  return (DIM == 3 ? 7 : 6) + (offdiag ? 4 : 0);
}

template <typename T, int DIM>
__device__ inline size_t level_elems(const Lvl<T>& a) {
  return DIM == 3 ? (size_t)a.S * (size_t)(a.mz + 3) : (size_t)a.P * (size_t)(a.my + 3);
}

template <typename T, int DIM>
__global__ void __launch_bounds__(512) k_coarse_staged(const LvlTable<T>* tab, CycleParams cp, int lev0, int fcycle,
                                                      int skip_pre, CoarseOps ops) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ LvlTable<T> st;        // the levels, pointers into shared memory
  __shared__ CoarseOps sops;        // the sub-cycle's operations
  __shared__ Lvl<T> top;            // the first coarse level in global memory
  __shared__ __align__(8) uint64_t bar;
  const int tid = threadIdx.x;
  {
    // the table was stored at the start of the solve, long before this launch
    const int n = (int)(sizeof(LvlTable<T>) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(tab);
    int* dst = reinterpret_cast<int*>(&st);
    for (int k = tid; k < n; k += blockDim.x) dst[k] = src[k];
  }
  stage_coarse_ops(ops, &sops);
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (tid == 0) {
    top = st.l[lev0];
    // shared-memory layout and the transfers of the constant arrays
    T* base = reinterpret_cast<T*>(smraw);
    // bytes the transfers bring: every coefficient array, phi and rhs of the first level
    // (the deeper levels' phi and rhs get space but no copy)
    uint32_t copied = 0;
    for (int l = lev0; l <= cp.last_level; ++l) {
      const size_t n = level_elems<T, DIM>(st.l[l]);
      const uint32_t b = (uint32_t)(n * sizeof(T));
      copied += (l == lev0 ? 2u : 0u) * b;
      copied += (uint32_t)(staged_arrays<T, DIM>(st.l[l].xll != nullptr) - 2) * b;
    }
    mbar_expect_tx(&bar, copied);
    for (int l = lev0; l <= cp.last_level; ++l) {
      Lvl<T>& v = st.l[l];
      const Lvl<T> g = v;
      const size_t n = level_elems<T, DIM>(g);
      const uint32_t b = (uint32_t)(n * sizeof(T));
      v.phi = base;
      v.rhs = base + n;
      T* q = base + 2 * n;
      v.wx = q;
      bulk_g2s(q, g.wx, b, &bar);
      q += n;
      v.wy = q;
      bulk_g2s(q, g.wy, b, &bar);
      q += n;
      if (DIM == 3) {
        v.wz = q;
        bulk_g2s(q, g.wz, b, &bar);
        q += n;
      }
      v.invd = q;
      bulk_g2s(q, g.invd, b, &bar);
      q += n;
      v.acc = q;
      bulk_g2s(q, g.acc, b, &bar);
      q += n;
      if (g.xll) {
        T* const* srcs[4] = {&g.xll, &g.xrl, &g.xlr, &g.xrr};
        T** dsts[4] = {&v.xll, &v.xrl, &v.xlr, &v.xrr};
        for (int k = 0; k < 4; ++k) {
          *dsts[k] = q;
          bulk_g2s(q, *srcs[k], b, &bar);
          q += n;
        }
      }
      v.phi2 = nullptr;
      base = q;
    }
  }
  __syncthreads();
  pdl_enter();  // phi and rhs of the first coarse level come from the preceding kernels
  if (tid == 0) {
    const size_t n = level_elems<T, DIM>(top);
    bulk_g2s(st.l[lev0].phi, top.phi, (uint32_t)(n * sizeof(T)), &bar);
    bulk_g2s(st.l[lev0].rhs, top.rhs, (uint32_t)(n * sizeof(T)), &bar);
  }
  const bool ok = mbar_wait(&bar, 0, kWaitPolls);
  if (!__syncthreads_and(ok)) {
    // the transfer did not complete: report it, poison the first level's phi, wait
    // (bounded) for the copies still in flight and give up
    if (tid == 0) atomicExch(const_cast<int*>(&tab->fault), 1);
    const size_t n = level_elems<T, DIM>(top);
    for (size_t k = tid; k < n; k += blockDim.x) top.phi[k] = T(__int_as_float(0x7fc00000));
    mbar_wait(&bar, 0, kWaitPolls);
    return;
  }
  if (sops.n > 0) blk_run<T, DIM>(&st, cp, &sops);
  else blk_cycle<T, DIM>(&st, cp, lev0, fcycle != 0, skip_pre != 0);
  // phi of the first coarse level back to global memory (the frame is zero in both)
  {
    const size_t n = level_elems<T, DIM>(top);
    const T* src = st.l[lev0].phi;
    for (size_t k = tid; k < n; k += blockDim.x) top.phi[k] = src[k];
  }
}

}  // namespace

// Shared-memory bytes the staged kernel needs from level lev0 down to last, 0 when the
// arrays do not fit in 200 KB.
size_t coarse_staged_bytes(int dim, const size_t* elems, int lev0, int last, size_t elem_size, bool offdiag) {
  size_t n = 0;
  for (int l = lev0; l <= last; ++l) n += elems[l];
  const size_t arrays = (dim == 3 ? 7 : 6) + (offdiag ? 4 : 0);
  const size_t b = n * arrays * elem_size;
  return b <= 200 * 1024 ? b : 0;
}

template <typename T>
int prepare_coarse_staged(int dim, size_t bytes) {
  cudaError_t e = dim == 2 ? cudaFuncSetAttribute(k_coarse_staged<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)bytes)
                           : cudaFuncSetAttribute(k_coarse_staged<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)bytes);
  return e == cudaSuccess ? 0 : 1;
}

template <typename T>
void launch_coarse_staged(int dim, const LvlTable<T>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                          size_t smem, int threads, cudaStream_t s) {
  const CoarseOps ops = coarse_ops(cp, lev, fcycle != 0, skip_pre != 0);
  if (dim == 2)
    launch_k(k_coarse_staged<T, 2>, dim3(1), dim3(threads), smem, s, tab, cp, lev, fcycle, skip_pre, ops);
  else
    launch_k(k_coarse_staged<T, 3>, dim3(1), dim3(threads), smem, s, tab, cp, lev, fcycle, skip_pre, ops);
}

template int prepare_coarse_staged<float>(int, size_t);
template int prepare_coarse_staged<double>(int, size_t);
template void launch_coarse_staged<float>(int, const LvlTable<float>*, const CycleParams&, int, int, int, size_t, int,
                                          cudaStream_t);
template void launch_coarse_staged<double>(int, const LvlTable<double>*, const CycleParams&, int, int, int, size_t, int,
                                           cudaStream_t);

}  // namespace jmg
