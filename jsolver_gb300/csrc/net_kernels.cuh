// net_kernels.cuh — kernels of the learned initial guess (a small U-Net), forward and backward.
//
// The network predicts phi0 from (log D_xx, log D_yy, lambda, rhs); it is the only tensor-
// core work of the project. Activations and weights are BF16 in NHWC layout (channels
// innermost, a multiple of 16), accumulation is FP32. A 3x3 convolution with zero padding
// is an implicit GEMM: M = output pixels, N = output channels, K = 9 taps x input channels.
//   k_conv3x3        forward (and, with transposed / flipped weights, the data gradient):
//                    mma.sync m16n8k16 BF16 -> FP32, operands staged in shared memory and
//                    fed with ldmatrix; bias + ReLU fused into the epilogue
//   k_conv3x3_wgrad  weight gradient dW_t = dY^T X_t per tap t (K = pixels), the same MMA
//                    with ldmatrix.trans operands, FP32 atomics across pixel chunks
// plus elementwise kernels (ReLU mask, 2x2 average pooling, nearest upsampling + skip,
// input preparation, MSE, Adam with FP32 master weights).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace jmgnet {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x2(unsigned& r0, unsigned& r1, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x2_t(unsigned& r0, unsigned& r1, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(smem_addr(p)));
}
__device__ __forceinline__ void mma16816(float* c, unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------------------------------
// forward convolution. Block: 4 warps, output tile of 8 rows x 16 columns of one image;
// warp w computes image rows 2w and 2w+1 (two m16 tiles) for all COUT channels. The block
// keeps the weights in shared memory and walks several tiles.
// ---------------------------------------------------------------------------------------

constexpr int kTH = 8, kTW = 16;            // output tile
constexpr int kIH = kTH + 2, kIW = kTW + 2; // input tile with the 3x3 halo

template <int CIN, int COUT>
struct ConvSmem {
  static constexpr int XS = CIN + 8;       // padded pixel stride (bank spread for ldmatrix)
  static constexpr int WS = 9 * CIN + 8;   // padded weight row
  static constexpr int bytes = (kIH * kIW * XS + COUT * WS) * 2;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3x3(const bf16* __restrict__ X, const bf16* __restrict__ Wt,
                                                 const float* __restrict__ bias, const bf16* __restrict__ mask,
                                                 bf16* __restrict__ Y, float* __restrict__ Y32, int N, int H, int W,
                                                 int relu) {
  using S = ConvSmem<CIN, COUT>;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  bf16* xs = reinterpret_cast<bf16*>(sm_raw);
  bf16* ws = xs + kIH * kIW * S::XS;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // weights [COUT][9*CIN] -> shared, 16-byte chunks
  for (int t = tid; t < COUT * (9 * CIN / 8); t += 128) {
    const int co = t / (9 * CIN / 8), c8 = t % (9 * CIN / 8);
    *reinterpret_cast<uint4*>(ws + co * S::WS + c8 * 8) = *reinterpret_cast<const uint4*>(Wt + (size_t)co * 9 * CIN + c8 * 8);
  }
  const int tiles_x = W / kTW, tiles_y = H / kTH;
  const int ntiles = N * tiles_x * tiles_y;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int n = tile / (tiles_x * tiles_y), rem = tile % (tiles_x * tiles_y);
    const int y0 = (rem / tiles_x) * kTH, x0 = (rem % tiles_x) * kTW;
    __syncthreads();  // previous tile's reads of xs are done (and the weights are in place)
    for (int t = tid; t < kIH * kIW * (CIN / 8); t += 128) {
      const int pix = t / (CIN / 8), c8 = t % (CIN / 8);
      const int yy = y0 - 1 + pix / kIW, xx = x0 - 1 + pix % kIW;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (yy >= 0 && yy < H && xx >= 0 && xx < W)
        v = *reinterpret_cast<const uint4*>(X + (((size_t)n * H + yy) * W + xx) * CIN + c8 * 8);
      *reinterpret_cast<uint4*>(xs + pix * S::XS + c8 * 8) = v;
    }
    __syncthreads();
    float acc[2][COUT / 8][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < COUT / 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.f;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int dh = tap / 3, dw = tap % 3;
#pragma unroll
      for (int c0 = 0; c0 < CIN; c0 += 16) {
        unsigned a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int r = warp * 2 + mt;  // output row within the tile
          const int px = (lane & 15);    // output column = A row
          const int col = c0 + ((lane >> 4) << 3);
          ldsm_x4(a[mt][0], a[mt][1], a[mt][2], a[mt][3], xs + ((r + dh) * kIW + px + dw) * S::XS + col);
        }
#pragma unroll
        for (int nt = 0; nt < COUT / 8; ++nt) {
          unsigned b0, b1;
          const int co = nt * 8 + (lane & 7);
          const int k = tap * CIN + c0 + (((lane >> 3) & 1) << 3);
          ldsm_x2(b0, b1, ws + co * S::WS + k);
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) mma16816(acc[mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
        }
      }
    }
    // epilogue: bias, ReLU, store (row of A = output column)
    const int g = lane >> 2, tg = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int yy = y0 + warp * 2 + mt;
#pragma unroll
      for (int nt = 0; nt < COUT / 8; ++nt) {
        const int co = nt * 8 + tg * 2;
        const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int xx = x0 + g + 8 * h;
          float v0 = acc[mt][nt][2 * h] + b0, v1 = acc[mt][nt][2 * h + 1] + b1;
          if (relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          const size_t o = (((size_t)n * H + yy) * W + xx) * COUT + co;
          if (mask) {  // gradient through a ReLU: zero where its output was not positive
            const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask + o);
            if (!(__low2float(mk) > 0.f)) v0 = 0.f;
            if (!(__high2float(mk) > 0.f)) v1 = 0.f;
          }
          if (Y32) {
            Y32[o] = v0;
            Y32[o + 1] = v1;
          } else {
            *reinterpret_cast<__nv_bfloat162*>(Y + o) = __floats2bfloat162_rn(v0, v1);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// weight gradient: dW[co][tap][ci] += sum_p dY[p][co] X[p + off(tap)][ci]. Grid: (tap,
// co block of 16, pixel chunk). Each warp takes two rows of a 8x16 tile (32 pixels = two
// k16 steps); the four warps' partial sums are combined in shared memory and added to
// dW with FP32 atomics.
// ---------------------------------------------------------------------------------------

template <int CIN, int COUT>
struct WgSmem {
  static constexpr int XS = CIN + 8;
  static constexpr int YS = COUT + 8;
  static constexpr int bytes = (kIH * kIW * XS + kTH * kTW * YS) * 2;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const bf16* __restrict__ X, const bf16* __restrict__ dY,
                                                       float* __restrict__ dW, int N, int H, int W, int chunks) {
  using S = WgSmem<CIN, COUT>;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  bf16* xs = reinterpret_cast<bf16*>(sm_raw);
  bf16* ys = xs + kIH * kIW * S::XS;
  __shared__ float red[4][16 * CIN];
  const int tap = blockIdx.x, mblk = blockIdx.y, chunk = blockIdx.z;
  const int dh = tap / 3, dw = tap % 3;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = W / kTW, tiles_y = H / kTH, ntiles = N * tiles_x * tiles_y;
  float acc[CIN / 8][4];
#pragma unroll
  for (int nt = 0; nt < CIN / 8; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
  for (int tile = chunk; tile < ntiles; tile += chunks) {
    const int n = tile / (tiles_x * tiles_y), rem = tile % (tiles_x * tiles_y);
    const int y0 = (rem / tiles_x) * kTH, x0 = (rem % tiles_x) * kTW;
    __syncthreads();
    for (int t = tid; t < kIH * kIW * (CIN / 8); t += 128) {
      const int pix = t / (CIN / 8), c8 = t % (CIN / 8);
      const int yy = y0 - 1 + pix / kIW, xx = x0 - 1 + pix % kIW;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (yy >= 0 && yy < H && xx >= 0 && xx < W)
        v = *reinterpret_cast<const uint4*>(X + (((size_t)n * H + yy) * W + xx) * CIN + c8 * 8);
      *reinterpret_cast<uint4*>(xs + pix * S::XS + c8 * 8) = v;
    }
    for (int t = tid; t < kTH * kTW * (COUT / 8); t += 128) {
      const int pix = t / (COUT / 8), c8 = t % (COUT / 8);
      const int yy = y0 + pix / kTW, xx = x0 + pix % kTW;
      *reinterpret_cast<uint4*>(ys + pix * S::YS + c8 * 8) =
          *reinterpret_cast<const uint4*>(dY + (((size_t)n * H + yy) * W + xx) * COUT + c8 * 8);
    }
    __syncthreads();
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int r = warp * 2 + rr;  // tile row: 16 pixels = one k16 step
      // A = dY^T (16 channels of this block x 16 pixels): four 8x8 blocks, transposed loads
      unsigned a0, a1, a2, a3;
      {
        const int px = ((lane >> 4) << 3) + (lane & 7);  // pixel 0-7 or 8-15
        const int co = mblk * 16 + (((lane >> 3) & 1) << 3);
        ldsm_x4_t(a0, a1, a2, a3, ys + (r * kTW + px) * S::YS + co);
      }
#pragma unroll
      for (int nt = 0; nt < CIN / 8; ++nt) {
        unsigned b0, b1;
        const int px = ((lane >> 3) & 1) * 8 + (lane & 7);  // pixel of the k row
        ldsm_x2_t(b0, b1, xs + ((r + dh) * kIW + px + dw) * S::XS + nt * 8);
        mma16816(acc[nt], a0, a1, a2, a3, b0, b1);
      }
    }
  }
  // combine the four warps, then one atomic per output element
  const int g = lane >> 2, tg = lane & 3;
#pragma unroll
  for (int nt = 0; nt < CIN / 8; ++nt)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int m = g + 8 * h;  // co within the block
      const int ci = nt * 8 + tg * 2;
      red[warp][m * CIN + ci] = acc[nt][2 * h];
      red[warp][m * CIN + ci + 1] = acc[nt][2 * h + 1];
    }
  __syncthreads();
  for (int t = tid; t < 16 * CIN; t += 128) {
    const float v = red[0][t] + red[1][t] + red[2][t] + red[3][t];
    const int m = t / CIN, ci = t % CIN;
    atomicAdd(&dW[((size_t)(mblk * 16 + m) * 9 + tap) * CIN + ci], v);
  }
}

// ---------------------------------------------------------------------------------------
// elementwise kernels (NHWC, C channels)
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ bool relu_on(const bf16* mask, size_t t) {
  return !mask || __bfloat162float(mask[t]) > 0.f;
}

// bias gradient: db[c] += sum over pixels of dY[p][c]
__global__ void k_bias_grad(const bf16* __restrict__ dY, float* __restrict__ db, size_t npix, int C) {
  const int c = blockIdx.y;
  float s = 0.f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x)
    s += __bfloat162float(dY[p * C + c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ float w[32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += w[i];
    atomicAdd(&db[c], t);
  }
}

// 2x2 average pooling (H, W even): Y = bf16(0.25 * (((x00 + x01) + x10) + x11))
__global__ void k_pool2(const bf16* __restrict__ X, bf16* __restrict__ Y, int N, int H, int W, int C) {
  const size_t n_out = (size_t)N * (H / 2) * (W / 2) * C;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n_out; t += (size_t)gridDim.x * blockDim.x) {
    const int c = t % C;
    size_t r = t / C;
    const int x = r % (W / 2);
    r /= (W / 2);
    const int y = r % (H / 2);
    const int n = r / (H / 2);
    auto at = [&](int yy, int xx) { return __bfloat162float(X[(((size_t)n * H + yy) * W + xx) * C + c]); };
    const float v = 0.25f * (((at(2 * y, 2 * x) + at(2 * y, 2 * x + 1)) + at(2 * y + 1, 2 * x)) + at(2 * y + 1, 2 * x + 1));
    Y[t] = __float2bfloat16(v);
  }
}

// gradient of 2x2 average pooling plus the skip gradient `add` (nullable), through the
// ReLU whose output is `mask` (nullable): dX = mask ? bf16(0.25 dY + add) : 0
__global__ void k_pool2_bwd(const bf16* __restrict__ dY, const bf16* __restrict__ add, const bf16* __restrict__ mask,
                            bf16* __restrict__ dX, int N, int H, int W, int C) {
  const size_t n_in = (size_t)N * H * W * C;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n_in; t += (size_t)gridDim.x * blockDim.x) {
    const int c = t % C;
    size_t r = t / C;
    const int x = r % W;
    r /= W;
    const int y = r % H;
    const int n = r / H;
    float v = 0.25f * __bfloat162float(dY[(((size_t)n * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c]);
    if (add) v += __bfloat162float(add[t]);
    dX[t] = __float2bfloat16(relu_on(mask, t) ? v : 0.f);
  }
}

// U = bf16(up2(Xc) + skip): nearest-neighbour upsampling of the coarse tensor plus the skip
__global__ void k_up2_add(const bf16* __restrict__ Xc, const bf16* __restrict__ skip, bf16* __restrict__ U, int N,
                          int H, int W, int C) {
  const size_t n_out = (size_t)N * H * W * C;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n_out; t += (size_t)gridDim.x * blockDim.x) {
    const int c = t % C;
    size_t r = t / C;
    const int x = r % W;
    r /= W;
    const int y = r % H;
    const int n = r / H;
    const float v = __bfloat162float(Xc[(((size_t)n * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c]) +
                    __bfloat162float(skip[t]);
    U[t] = __float2bfloat16(v);
  }
}

// gradient of up2 through the ReLU whose output is `mask`: dXc = bf16(((g00 + g01) + g10) + g11)
__global__ void k_up2_bwd(const bf16* __restrict__ dU, const bf16* __restrict__ mask, bf16* __restrict__ dXc, int N,
                          int H, int W, int C) {
  const size_t n_out = (size_t)N * (H / 2) * (W / 2) * C;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n_out; t += (size_t)gridDim.x * blockDim.x) {
    const int c = t % C;
    size_t r = t / C;
    const int x = r % (W / 2);
    r /= (W / 2);
    const int y = r % (H / 2);
    const int n = r / (H / 2);
    auto at = [&](int yy, int xx) { return __bfloat162float(dU[(((size_t)n * H + yy) * W + xx) * C + c]); };
    const float v = ((at(2 * y, 2 * x) + at(2 * y, 2 * x + 1)) + at(2 * y + 1, 2 * x)) + at(2 * y + 1, 2 * x + 1);
    dXc[t] = __float2bfloat16(relu_on(mask, t) ? v : 0.f);
  }
}

// mean squared error of channel 0 of the FP32 output against the target; writes the
// output gradient (bf16, 16 channels, zero beyond channel 0) and adds the loss / npix
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target, bf16* __restrict__ grad,
                      float* __restrict__ loss, size_t npix) {
  const float inv = 1.f / (float)npix;
  float s = 0.f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
    const float d = pred[p * 16] - target[p];
    s += d * d;
    uint4 z[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    bf16* zb = reinterpret_cast<bf16*>(z);
    zb[0] = __float2bfloat16(2.f * d * inv);
    uint4* g = reinterpret_cast<uint4*>(grad + p * 16);
    g[0] = z[0];
    g[1] = z[1];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv);
}

// channel 0 of the FP32 output -> dense [npix]
__global__ void k_take_channel0(const float* __restrict__ y32, float* __restrict__ y, size_t npix) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x)
    y[p] = y32[p * 16];
}

// Adam (bias-corrected, FP32 master weights)
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[t];
    const float mi = b1 * m[t] + (1.f - b1) * gi;
    const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
    m[t] = mi;
    v[t] = vi;
    w[t] = w[t] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// BF16 copies of one layer's FP32 weights [cout][9][cin]: wb in the same layout, wt
// transposed and flipped, [cin][9][cout] at tap 8 - t (the data-gradient convolution)
__global__ void k_pack_weights(const float* __restrict__ w, bf16* __restrict__ wb, bf16* __restrict__ wt, int cout,
                               int cin) {
  const int n = cout * 9 * cin;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ci = t % cin, tp = (t / cin) % 9, co = t / (9 * cin);
    const bf16 b = __float2bfloat16(w[t]);
    wb[t] = b;
    wt[((size_t)ci * 9 + (8 - tp)) * cout + co] = b;
  }
}

}  // namespace jmgnet
