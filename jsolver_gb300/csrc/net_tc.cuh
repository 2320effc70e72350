// net_tc.cuh — the 3x3 convolution of the learned guess on the 5th-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory, operands staged by TMA).
//
// Implicit GEMM per 8 x 16 output tile: D[128 pixels][COUT] = sum over 9 taps and CIN/16
// K-steps of A_tap[128 pixels][16 channels] x B_tap[COUT][16 channels]^T, BF16 operands,
// FP32 accumulation in TMEM (128 lanes = pixels, COUT columns).
//   A: the input tile with its one-pixel halo arrives by TMA (cp.async.bulk.tensor.4d on
//      the NHWC activation, zero fill outside the image) as three copies shifted by
//      dw = 0, 1, 2 columns, each [CIN/8 channel planes][10 rows][16 columns][8 channels].
//      For tap (dh, dw) the 128 rows of A are rows dh .. dh+7 of copy dw: 8 consecutive
//      pixels of one plane form a core matrix (8 rows x 16 bytes, contiguous), the next 8
//      pixels follow at 128 bytes (stride byte offset) and the next 8 channels one plane
//      further (leading byte offset): the canonical K-major layout without swizzle.
//   B: the weights [COUT][9][CIN] rearranged once per block into [tap][CIN/8][COUT][8]:
//      core matrices of 8 output channels x 8 input channels, 128 bytes apart along N,
//      one [COUT][8] plane apart along K.
// One thread issues the MMAs and commits them to an mbarrier; after the wait every warp
// reads its 32 TMEM lanes (tcgen05.ld 32x32b) and applies bias, ReLU / the gradient mask
// and the store, as the mma.sync kernel's epilogue does. Two input stages and two
// accumulators let the loads of the next tile, the MMAs of the current one and the
// epilogue of the previous one overlap. Every wait is bounded: on a timeout the block
// raises *fault, stops taking tiles, waits (bounded) for what is in flight and releases
// its tensor memory.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace jmgnet {

constexpr long long kTcPolls = 1LL << 22;

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tc_mbar_init(uint64_t* bar, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(tc_smem(bar)), "r"(n) : "memory");
}

__device__ __forceinline__ bool tc_mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = tc_smem(bar);
  for (long long k = 0; k < kTcPolls; ++k) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// shared-memory matrix descriptor: K-major, no swizzle (start, leading and stride byte
// offsets in 16-byte units, descriptor version 1)
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N, M
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <int CIN, int COUT>
struct TcConv {
  static constexpr int APLANE = kIH * kTW * 16;        // one [10][16][8] channel plane, bytes
  static constexpr int ASTAGE = 3 * (CIN / 8) * APLANE; // one input tile (three shifted copies)
  static constexpr int BPLANE = COUT * 16;              // one [COUT][8] plane, bytes
  static constexpr int BBYTES = 9 * (CIN / 8) * BPLANE;
  static constexpr int smem = 2 * ASTAGE + BBYTES + 128;  // two input stages, + alignment slack
  static constexpr int ACOLS = COUT < 32 ? 32 : COUT;     // one accumulator's TMEM columns
  static constexpr int TCOLS = 2 * ACOLS;                 // two accumulators (a power of 2)
};

// issue the TMA loads of one input tile (three column-shifted copies of every plane)
template <int CIN>
__device__ __forceinline__ void tc_load_tile(const CUtensorMap* xmap, unsigned char* A, int aplane, int n, int y0,
                                             int x0, uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(tc_smem(bar)), "r"(bytes) : "memory");
  for (int dw = 0; dw < 3; ++dw)
    for (int c8 = 0; c8 < CIN / 8; ++c8) {
      unsigned char* dst = A + (dw * (CIN / 8) + c8) * aplane;
      asm volatile(
          "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
          "%5}], [%6];\n" ::"r"(tc_smem(dst)),
          "l"(reinterpret_cast<uint64_t>(xmap)), "r"(c8 * 8), "r"(x0 - 1 + dw), "r"(y0 - 1), "r"(n), "r"(tc_smem(bar))
          : "memory");
    }
}

// The tiles of a block run as a two-stage pipeline: while every warp reads tile i-1's
// accumulator out of tensor memory, the tensor cores work on tile i (the other
// accumulator) and the TMA engine loads tile i+1 (the other input stage).
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3x3_tc(const __grid_constant__ CUtensorMap xmap,
                                                    const bf16* __restrict__ Wt, const float* __restrict__ bias,
                                                    const bf16* __restrict__ mask, bf16* __restrict__ Y,
                                                    float* __restrict__ Y32, int N, int H, int W, int relu,
                                                    int* __restrict__ fault) {
  using S = TcConv<CIN, COUT>;
  extern __shared__ unsigned char sm_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sm_raw) + 127) & ~uintptr_t(127));
  unsigned char* Bs = base + 2 * S::ASTAGE;
  __shared__ __align__(8) uint64_t bar_tma[2], bar_mma[2];
  __shared__ uint32_t tmem_base;
  __shared__ int stop;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc_smem(&tmem_base)),
                 "r"(S::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int k = 0; k < 2; ++k) {
      tc_mbar_init(&bar_tma[k], 1);
      tc_mbar_init(&bar_mma[k], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    stop = 0;
  }
  // weights [COUT][9][CIN] -> [tap][CIN/8][COUT][8]
  for (int t = tid; t < COUT * 9 * (CIN / 8); t += 128) {
    const int co = t / (9 * (CIN / 8)), r = t % (9 * (CIN / 8));
    const int tap = r / (CIN / 8), c8 = r % (CIN / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(Wt + ((size_t)co * 9 + tap) * CIN + c8 * 8);
    *reinterpret_cast<uint4*>(Bs + (tap * (CIN / 8) + c8) * S::BPLANE + co * 16) = v;
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // visible to the tensor cores
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = tc_idesc(128, COUT);
  const int tiles_x = W / kTW, tiles_y = H / kTH;
  const int ntiles = N * tiles_x * tiles_y;
  const int mine = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;  // tiles of this block
  auto tile_at = [&](int k, int& n, int& y0, int& x0) {
    const int tile = blockIdx.x + k * gridDim.x;
    n = tile / (tiles_x * tiles_y);
    const int rem = tile % (tiles_x * tiles_y);
    y0 = (rem / tiles_x) * kTH;
    x0 = (rem % tiles_x) * kTW;
  };
  if (tid == 0 && mine > 0) {
    int n, y0, x0;
    tile_at(0, n, y0, x0);
    tc_load_tile<CIN>(&xmap, base, S::APLANE, n, y0, x0, &bar_tma[0], S::ASTAGE);
  }
  // the epilogue of the k-th tile of the block (accumulator k % 2)
  auto epilogue = [&](int k) {
    int n, y0, x0;
    tile_at(k, n, y0, x0);
    const uint32_t acc = tmem + (uint32_t)((k & 1) * S::ACOLS);
    const int m = warp * 32 + lane;  // warp w holds TMEM lanes 32w .. 32w+31 = pixels of the tile
    const int yy = y0 + (m >> 4), xx = x0 + (m & 15);
    const size_t o = (((size_t)n * H + yy) * W + xx) * COUT;
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = acc + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      float v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        v[q] = __uint_as_float(r[q]) + (bias ? bias[c0 + q] : 0.f);
        if (relu) v[q] = fmaxf(v[q], 0.f);
      }
      if (mask) {  // gradient through a ReLU: zero where its output was not positive
        const uint4* mk = reinterpret_cast<const uint4*>(mask + o + c0);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint4 w4 = mk[h];
          const bf16* mb = reinterpret_cast<const bf16*>(&w4);
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (!(__bfloat162float(mb[q]) > 0.f)) v[8 * h + q] = 0.f;
        }
      }
      if (Y32) {
#pragma unroll
        for (int q = 0; q < 16; q += 4)
          *reinterpret_cast<float4*>(Y32 + o + c0 + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
      } else {
        uint4 w4[2];
        __nv_bfloat162* wb = reinterpret_cast<__nv_bfloat162*>(w4);
#pragma unroll
        for (int q = 0; q < 8; ++q) wb[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
        *reinterpret_cast<uint4*>(Y + o + c0) = w4[0];
        *reinterpret_cast<uint4*>(Y + o + c0 + 8) = w4[1];
      }
    }
  };
  int k = 0;
  for (; k < mine; ++k) {
    const int st = k & 1;
    if (tid == 0) {
      bool ok = true;
      // tile k-1's MMAs are done: its input stage takes tile k+1
      if (k >= 1) ok = tc_mbar_wait(&bar_mma[st ^ 1], ((k - 1) >> 1) & 1);
      if (ok && k + 1 < mine) {
        int n, y0, x0;
        tile_at(k + 1, n, y0, x0);
        tc_load_tile<CIN>(&xmap, base + (st ^ 1) * S::ASTAGE, S::APLANE, n, y0, x0, &bar_tma[st ^ 1], S::ASTAGE);
      }
      if (ok) ok = tc_mbar_wait(&bar_tma[st], (k >> 1) & 1);
      if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const unsigned char* A = base + st * S::ASTAGE;
        const uint32_t acc = tmem + (uint32_t)(st * S::ACOLS);
        int first = 1;
        for (int tap = 0; tap < 9; ++tap) {
          const int dh = tap / 3, dw = tap % 3;
          for (int kc = 0; kc < CIN / 16; ++kc) {
            const uint32_t a = tc_smem(A + (dw * (CIN / 8) + 2 * kc) * S::APLANE + dh * kTW * 16);
            const uint32_t b = tc_smem(Bs + (tap * (CIN / 8) + 2 * kc) * S::BPLANE);
            const uint64_t ad = tc_desc(a, S::APLANE, 128), bd = tc_desc(b, S::BPLANE, 128);
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
                "l"(ad), "l"(bd), "r"(idesc), "r"(first ? 0 : 1)
                : "memory");
            first = 0;
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         tc_smem(&bar_mma[st]))
                     : "memory");
      } else {
        atomicExch(fault, 1);
        stop = 1;
      }
    }
    __syncthreads();
    if (stop) break;
    if (k >= 1) {
      const bool done = tc_mbar_wait(&bar_mma[st ^ 1], ((k - 1) >> 1) & 1);
      if (!__syncthreads_and(done)) {
        if (tid == 0) atomicExch(fault, 1);
        stop = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      epilogue(k - 1);
    }
    // the accumulator just read out takes tile k+1's MMAs after this barrier
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
  }
  if (!stop && mine > 0) {
    const int last = mine - 1;
    const bool done = tc_mbar_wait(&bar_mma[last & 1], (last >> 1) & 1);
    if (__syncthreads_and(done)) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      epilogue(last);
    } else if (tid == 0) {
      atomicExch(fault, 1);
    }
  } else if (stop) {
    // a transfer or the tensor cores did not answer: wait (bounded) for what may still
    // be in flight before the tensor memory is released
    tc_mbar_wait(&bar_tma[k & 1], (k >> 1) & 1);
    tc_mbar_wait(&bar_mma[k & 1], (k >> 1) & 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::TCOLS) : "memory");
}

}  // namespace jmgnet
