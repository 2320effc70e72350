// mg_mid2d.cu — the middle and coarse levels of a 2D cycle in one cooperative launch.
//
// Below the finest level a 2D cycle is bound by launch latency, not by bytes: every visit
// of a grid-wide level runs two fused launches (smooth + restrict, prolong + smooth,
// mg_fusedops2d.cuh) of a few microseconds each, and the coarse sub-cycle one more. Here
// the part of the recursion (solver_2d.py:582-614) from level `lev0` down runs as one
// persistent kernel with one block per SM:
//   * grid-wide operations are the same tiles as the fused kernels, spread over the blocks,
//     each followed by a grid barrier instead of a kernel boundary;
//   * the coarse sub-cycle (levels of at most a few thousand points) runs on block 0 over
//     the shared-memory copies of its levels (mg_block.cuh's single-block operators) while
//     the other blocks wait at the next barrier. Block 0 stages the coarse coefficients
//     once per launch, with bulk copies issued at kernel entry, so a W-cycle's many coarse
//     visits share one transfer.
// The host builds the operation list in the order of the reference's recursion (V, W, F;
// extra sweeps as colour passes), and every value is computed by the per-point functions
// of the other kernels in the same order, so results are bit-identical to the launches
// this kernel replaces.
//
// Memory: phi and rhs, which other blocks of the launch write, are read through L2 only
// (ld.global.cg); coefficient arrays are constant during a solve. The barrier is
// generation-based: thread 0 of each block reads the generation, adds itself to the
// arrival count (release), and the last arrival resets the count and bumps the generation;
// the others poll the generation (acquire). Co-residency of all blocks comes from the
// cooperative launch. Every wait is bounded: a barrier (or block 0's wait for its staging
// copies) that runs out sets the loop state's fault flag, the blocks fill the level's phi
// with NaN and return, and the loop-step kernel ends the solve (jmg_solve_check reports
// JMG_ERR_TIMEOUT).
#include <cuda_runtime.h>

#include <cstdint>

#include "mg_block.cuh"
#include "mg_bulk.cuh"
#include "mg_common.cuh"
#include "mg_fusedops2d.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

constexpr int kMidThreads = 512;  // the tile functions below are instantiated for it
constexpr long long kBarrierPolls = 1LL << 22;  // an L2 round trip and a short sleep each: a second or two
constexpr long long kStallPolls = 2000;         // test mode: the barrier can never complete

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier over `expect` arrivals; false when the wait ran out (fault flag set).
__device__ bool grid_barrier(LoopState* st, unsigned expect, long long polls, int* ok_s) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = ld_acquire(&st->bar_gen);
    __threadfence();
    const unsigned arrived = atomicAdd(&st->bar_count, 1u) + 1u;
    if (arrived == expect) {
      atomicExch(&st->bar_count, 0u);
      __threadfence();
      st_release(&st->bar_gen, g + 1u);
    } else {
      long long k = 0;
      while (ld_acquire(&st->bar_gen) == g) {
        if (++k > polls) {
          ok = 0;
          atomicExch(&st->fault, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    *ok_s = ok;
  }
  __syncthreads();
  return *ok_s != 0;
}

// One colour pass of a level in place, over the whole grid (gs_point2d's order).
template <typename T>
__device__ __forceinline__ void color_pass(const Lvl<T>& a, int color) {
  const int hx = a.mx / 2, sh = log2_pow2(hx);
  const int n = hx * (a.my - 1);
  const int P = a.P;
  T* __restrict__ ph = a.phi;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 2 + (t >> sh);
    const int j = 2 + ((i + color) & 1) + 2 * (t & (hx - 1));
    if (j > a.mx) continue;
    const long long p = (long long)i * P + j;
    T s = a.wy[p] * __ldcg(ph + p + P);
    s = fma(a.wy[p - P], __ldcg(ph + p - P), s);
    s = fma(a.wx[p], __ldcg(ph + p + 1), s);
    s = fma(a.wx[p - 1], __ldcg(ph + p - 1), s);
    s = s - __ldcg(a.rhs + p);
    ph[p] = s * a.invd[p];
  }
}

template <typename T>
__device__ inline size_t elems2d(const Lvl<T>& a) {
  return (size_t)a.P * (size_t)(a.my + 3);
}

// The operations as separate (not inlined) functions, so that each gets its own register
// allocation instead of the union of all of them in one kernel body.
template <typename T>
__device__ __noinline__ void op_smooth_restrict(const Lvl<T>& f, const Lvl<T>& c, int zero_in,
                                                unsigned char* smraw) {
  using F = FusedShape<T>;
  const int gx = (c.mx + 3 + F::CI - 1) / F::CI, gy = (c.my + 3 + F::CJ - 1) / F::CJ;
  for (int t = blockIdx.x; t < gx * gy; t += gridDim.x) {
    smooth_restrict_tile<T, F::CJ, F::CI, 512, true>(f, f.phi2, c, zero_in, t / gx, t % gx, smraw);
    __syncthreads();
  }
}

// f: the level with its two phi views swapped (phi = the smoothed phi of the restriction,
// phi2 = the buffer to write)
template <typename T>
__device__ __noinline__ void op_prolong_smooth(const Lvl<T>& f, const Lvl<T>& c, unsigned char* smraw) {
  using F = FusedShape<T>;
  const int gx = (f.mx - 1 + F::TI - 1) / F::TI, gy = (f.my - 1 + F::TJ - 1) / F::TJ;
  for (int t = blockIdx.x; t < gx * gy; t += gridDim.x) {
    prolong_smooth_tile<T, F::TJ, F::TI, 512, true>(f, f.phi2, c, t / gx, t % gx, smraw);
    __syncthreads();
  }
}

template <typename T>
__device__ __noinline__ void op_block(int kind, const Lvl<T>& a, const Lvl<T>& c, int diag) {
  if (kind == kMidBlkSweep) blk_sweep<T, 2>(a);
  else if (kind == kMidBlkRestrict) blk_restrict<T, 2>(a, c);
  else blk_prolong<T, 2>(a, c, diag != 0);
}

template <typename T>
__global__ void __launch_bounds__(kMidThreads, 1)
    k_mid_cycle2d(const LvlTable<T>* tab, LoopState* st, CycleParams cp, int cs, unsigned expect, long long polls,
                  int tile_bytes, MidOps ops) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ LvlTable<T> gt;  // the levels in global memory (canonical phi buffers)
  __shared__ LvlTable<T> bt;  // block 0: the coarse levels in shared memory
  __shared__ Lvl<T> pf;        // the level a prolong + smooth tile works on (buffers swapped)
  __shared__ __align__(8) uint64_t bar;
  __shared__ int ok_s;
  const int tid = threadIdx.x;
  const bool b0 = blockIdx.x == 0;
  {
    // the table was stored at the start of the solve, long before this launch
    const int n = (int)(sizeof(LvlTable<T>) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(tab);
    int* dst = reinterpret_cast<int*>(&gt);
    for (int k = tid; k < n; k += blockDim.x) dst[k] = src[k];
  }
  if (b0 && tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (b0 && tid == 0) {
    // block 0: coarse coefficients into shared memory behind the tile area (the cycle
    // never writes them); phi and rhs of each coarse level get space, no copy
    uint32_t copied = 0;
    for (int l = cs; l <= cp.last_level; ++l) copied += 4u * (uint32_t)(elems2d(gt.l[l]) * sizeof(T));
    mbar_expect_tx(&bar, copied);
    T* base = reinterpret_cast<T*>(smraw + tile_bytes);
    for (int l = 0; l < kMaxLevels; ++l) bt.l[l] = gt.l[l];
    for (int l = cs; l <= cp.last_level; ++l) {
      Lvl<T>& v = bt.l[l];
      const Lvl<T>& g = gt.l[l];
      const size_t n = elems2d(g);
      const uint32_t b = (uint32_t)(n * sizeof(T));
      v.phi = base;
      v.rhs = base + n;
      v.wx = base + 2 * n;
      v.wy = base + 3 * n;
      v.invd = base + 4 * n;
      v.acc = base + 5 * n;
      v.phi2 = nullptr;
      bulk_g2s(v.wx, g.wx, b, &bar);
      bulk_g2s(v.wy, g.wy, b, &bar);
      bulk_g2s(v.invd, g.invd, b, &bar);
      bulk_g2s(v.acc, g.acc, b, &bar);
      base += 6 * n;
    }
  }
  pdl_enter();
  __syncthreads();
  bool staged = false;  // block 0 has waited for its staging copies
  bool in_blk = false;  // inside a run of block-0 operations
  bool ok = true;
  for (int o = 0; o < ops.n && ok; ++o) {
    const unsigned op = ops.op[o];
    const int kind = (int)(op >> 12), flag = (int)((op >> 8) & 1), lev = (int)(op & 31);
    if (kind <= kMidBlkProlong) {
      if (b0) {
        if (!in_blk) {
          if (!staged) {
            staged = true;
            if (!__syncthreads_and(mbar_wait(&bar, 0, kWaitPolls))) {
              if (tid == 0) atomicExch(&st->fault, 1);
              mbar_wait(&bar, 0, kWaitPolls);  // (bounded) for the copies still in flight
              ok = false;
              break;
            }
          }
          // phi and rhs of the first coarse level, written by the restriction above
          const Lvl<T>& g = gt.l[cs];
          const Lvl<T>& v = bt.l[cs];
          const int n = (int)elems2d(g);
          for (int k = tid; k < n; k += blockDim.x) {
            const T a = __ldcg(g.phi + k), r = __ldcg(g.rhs + k);
            v.phi[k] = a;
            v.rhs[k] = r;
          }
          __syncthreads();
        }
        op_block<T>(kind, bt.l[lev], bt.l[lev + 1], cp.diag);
      }
      in_blk = true;
      continue;
    }
    if (in_blk) {
      in_blk = false;
      if (b0) {
        // phi of the first coarse level back to global memory (frames are zero in both)
        const Lvl<T>& g = gt.l[cs];
        const T* src = bt.l[cs].phi;
        const int n = (int)elems2d(g);
        for (int k = tid; k < n; k += blockDim.x) g.phi[k] = src[k];
      }
      if (!(ok = grid_barrier(st, expect, polls, &ok_s))) break;
    }
    // the tiles read the level views from shared memory (registers stay for the tiles)
    if (kind == kMidSR) {
      op_smooth_restrict<T>(gt.l[lev], gt.l[lev + 1], flag, smraw);
    } else if (kind == kMidPS) {
      // the smoothed phi of the restriction is in the second buffer: swap the two views
      if (tid == 0) {
        pf = gt.l[lev];
        pf.phi = gt.l[lev].phi2;
        pf.phi2 = gt.l[lev].phi;
      }
      __syncthreads();
      op_prolong_smooth<T>(pf, gt.l[lev + 1], smraw);
    } else {
      color_pass<T>(gt.l[lev], flag);
    }
    if (o + 1 < ops.n && !(ok = grid_barrier(st, expect, polls, &ok_s))) break;
  }
  if (!ok) {
    // a wait ran out: the result of this launch is void; mark it in the first level's phi
    const Lvl<T>& a = gt.l[ops.n > 0 ? (ops.op[0] & 31) : 0];
    const int n = (int)elems2d(a);
    for (int k = blockIdx.x * blockDim.x + tid; k < n; k += gridDim.x * blockDim.x)
      a.phi[k] = T(__int_as_float(0x7fc00000));
  }
  // block 0 never leaves with bulk copies still landing in its shared memory
  if (b0 && !staged) mbar_wait(&bar, 0, kWaitPolls);
}

template <typename T>
size_t tile_bytes() {
  using F = FusedShape<T>;
  const size_t a = SR<T, F::CJ, F::CI>::smem, b = PS<T, F::TJ, F::TI>::smem;
  return ((a > b ? a : b) + 127) / 128 * 128;
}

void push(MidOps& o, int kind, int flag, int lev) {
  if (o.n >= 0 && o.n < kMaxMidOps) o.op[o.n++] = (unsigned short)((kind << 12) | (flag << 8) | lev);
  else o.n = -1;
}

// the coarse sub-cycle from lev (coarse_ops_rec's schedule, block-0 operations)
void blk_rec(const CycleParams& cp, int lev, bool fcycle, MidOps& o) {
  if (lev == cp.last_level) {
    for (int k = 0; k < cp.nu1 + cp.nu2; ++k) push(o, kMidBlkSweep, 0, lev);
    return;
  }
  for (int k = 0; k < cp.nu1; ++k) push(o, kMidBlkSweep, 0, lev);
  push(o, kMidBlkRestrict, 0, lev);
  if (fcycle)
    for (int g = 0; g < cp.gamma; ++g) blk_rec(cp, lev + 1, true, o);
  for (int g = 0; g < cp.gamma; ++g) blk_rec(cp, lev + 1, false, o);
  push(o, kMidBlkProlong, 0, lev);
  for (int k = 0; k < cp.nu2; ++k) push(o, kMidBlkSweep, 0, lev);
}

// a fused grid-wide level (emit_cycle's schedule with fused pairs), nu1, nu2 >= 1
void mid_rec(const CycleParams& cp, int cs, int lev, bool fcycle, bool zero_phi, MidOps& o) {
  if (lev >= cs) {
    blk_rec(cp, lev, fcycle, o);
    return;
  }
  for (int k = 0; k < cp.nu1 - 1; ++k) {
    push(o, kMidColor, 0, lev);
    push(o, kMidColor, 1, lev);
  }
  push(o, kMidSR, cp.nu1 == 1 && zero_phi ? 1 : 0, lev);
  bool first = true;
  if (fcycle)
    for (int g = 0; g < cp.gamma; ++g) {
      mid_rec(cp, cs, lev + 1, true, first, o);
      first = false;
    }
  for (int g = 0; g < cp.gamma; ++g) {
    mid_rec(cp, cs, lev + 1, false, first, o);
    first = false;
  }
  push(o, kMidPS, 0, lev);
  for (int k = 0; k < cp.nu2 - 1; ++k) {
    push(o, kMidColor, 0, lev);
    push(o, kMidColor, 1, lev);
  }
}

}  // namespace

bool mid_ops(const CycleParams& cp, int coarse_start, int lev, bool fcycle, bool zero_phi, MidOps* out) {
  out->n = 0;
  mid_rec(cp, coarse_start, lev, fcycle, zero_phi, *out);
  return out->n > 0;
}

template <typename T>
size_t prepare_mid2d(size_t staged_bytes, int* blocks) {
  *blocks = 0;
  int dev = 0, coop = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return 0;
  const size_t smem = tile_bytes<T>() + staged_bytes;
  if (cudaFuncSetAttribute(k_mid_cycle2d<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mid_cycle2d<T>, kMidThreads, smem) != cudaSuccess ||
      per_sm < 1)
    return 0;
  *blocks = sms;  // one block per SM, all resident
  return smem;
}

template <typename T>
cudaError_t launch_mid2d(const LvlTable<T>* tab, LoopState* st, const CycleParams& cp, int coarse_start,
                         const MidOps& ops, size_t smem, int blocks, bool stall, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kMidThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // test mode: one arrival more than there are blocks, so the first barrier runs out
  const unsigned expect = (unsigned)blocks + (stall ? 1u : 0u);
  const long long polls = stall ? kStallPolls : kBarrierPolls;
  return cudaLaunchKernelEx(&cfg, k_mid_cycle2d<T>, tab, st, cp, coarse_start, expect, polls,
                            (int)tile_bytes<T>(), ops);
}

template size_t prepare_mid2d<float>(size_t, int*);
template size_t prepare_mid2d<double>(size_t, int*);
template cudaError_t launch_mid2d<float>(const LvlTable<float>*, LoopState*, const CycleParams&, int,
                                         const MidOps&, size_t, int, bool, cudaStream_t);
template cudaError_t launch_mid2d<double>(const LvlTable<double>*, LoopState*, const CycleParams&, int,
                                          const MidOps&, size_t, int, bool, cudaStream_t);

}  // namespace jmg
