// mg_net.cu — the learned initial guess: U-Net runner, training step and the C ABI.
//
// The network (4 levels, 16/32/64/64 channels, 3x3 convolutions, ReLU, additive skips,
// 2x2 average pooling, nearest upsampling) maps four input channels on a res x res grid
// (log D_xx, log D_yy, lambda / 10, rhs / rms(rhs)) to phi0 / (out_scale * rms(rhs)).
// Layers (input -> output, level = resolution res / 2^level):
//   L0  x  -> a0   16->16 @0      L6  p2 = pool(a5) -> a6  64->64 @3
//   L1  a0 -> a1   16->16 @0      L7  a6 -> a7   64->64 @3
//   L2  p0 = pool(a1) -> a2 16->32 @1   L8  u2 = up(a7) + a5 -> a8  64->32 @2
//   L3  a2 -> a3   32->32 @1      L9  u1 = up(a8) + a3 -> a9  32->16 @1
//   L4  p1 = pool(a3) -> a4 32->64 @2   L10 u0 = up(a9) + a1 -> a10 16->16 @0
//   L5  a4 -> a5   64->64 @2      L11 a10 -> y (FP32, linear) 16->16 @0, channel 0 used
// Parameters (FP32 master copy) are stored layer by layer: weights [cout][3][3][cin],
// then the bias [cout]. Activations and activation gradients are BF16 (NHWC); every
// convolution accumulates in FP32 on the tensor cores (net_kernels.cuh).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/jmg.h"
#include "mg_kernels.h"
#include "net_kernels.cuh"
#include "net_tc.cuh"

using jmgnet::bf16;

namespace {

struct LayerDesc {
  int cin, cout, lev, relu;
};
constexpr int kLayers = 12;
constexpr LayerDesc kNet[kLayers] = {{16, 16, 0, 1}, {16, 16, 0, 1}, {16, 32, 1, 1}, {32, 32, 1, 1},
                                     {32, 64, 2, 1}, {64, 64, 2, 1}, {64, 64, 3, 1}, {64, 64, 3, 1},
                                     {64, 32, 2, 1}, {32, 16, 1, 1}, {16, 16, 0, 1}, {16, 16, 0, 0}};

size_t w_off(int l) {
  size_t o = 0;
  for (int k = 0; k < l; ++k) o += (size_t)kNet[k].cout * 9 * kNet[k].cin + kNet[k].cout;
  return o;
}
size_t num_params() { return w_off(kLayers); }
size_t w_elems(int l) { return (size_t)kNet[l].cout * 9 * kNet[l].cin; }

int grid_for(size_t n, int threads = 256) {
  size_t b = (n + threads - 1) / threads;
  const size_t cap = 152 * 16;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// ---- convolution dispatch ----------------------------------------------------------------

// The convolutions run on the tcgen05 kernel (net_tc.cuh) unless JMG_CONV=mma selects the
// mma.sync kernel (net_kernels.cuh), which the tests compare it with.
bool use_tcgen05() {
  const char* e = getenv("JMG_CONV");
  return !(e && std::strcmp(e, "mma") == 0);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// tensor map of an NHWC BF16 activation [N][H][W][C]: boxes of 8 channels x 16 columns x
// 10 rows of one image (an input tile with its halo, one 8-channel plane), zero fill
bool activation_map(CUtensorMap* m, const bf16* X, int N, int H, int W, int C) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t box[4] = {8, (cuuint32_t)jmgnet::kTW, (cuuint32_t)jmgnet::kIH, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(X), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int CIN, int COUT>
void conv_t(const bf16* X, const bf16* W, const float* bias, const bf16* mask, bf16* Y, float* Y32, int N, int H,
            int Wd, int relu, int* fault, cudaStream_t s) {
  const int tiles = N * (H / jmgnet::kTH) * (Wd / jmgnet::kTW);
  CUtensorMap xmap;
  if (use_tcgen05() && activation_map(&xmap, X, N, H, Wd, CIN)) {
    using S = jmgnet::TcConv<CIN, COUT>;
    // blocks per SM that shared memory (220 KB) and tensor memory (512 columns) allow
    int per_sm = (220 * 1024) / S::smem;
    if (per_sm > 512 / S::TCOLS) per_sm = 512 / S::TCOLS;
    if (per_sm < 1) per_sm = 1;
    const int blocks = tiles < 152 * per_sm ? tiles : 152 * per_sm;
    jmgnet::k_conv3x3_tc<CIN, COUT><<<blocks, 128, S::smem, s>>>(xmap, W, bias, mask, Y, Y32, N, H, Wd, relu, fault);
    return;
  }
  using S = jmgnet::ConvSmem<CIN, COUT>;
  const int blocks = tiles < 152 * 4 ? tiles : 152 * 4;
  jmgnet::k_conv3x3<CIN, COUT><<<blocks, 128, S::bytes, s>>>(X, W, bias, mask, Y, Y32, N, H, Wd, relu);
}

template <int CIN, int COUT>
void wgrad_t(const bf16* X, const bf16* dY, float* dW, int N, int H, int Wd, cudaStream_t s) {
  using S = jmgnet::WgSmem<CIN, COUT>;
  const int tiles = N * (H / jmgnet::kTH) * (Wd / jmgnet::kTW);
  int chunks = 2048 / (9 * (COUT / 16));
  if (chunks > tiles) chunks = tiles;
  if (chunks < 1) chunks = 1;
  jmgnet::k_conv3x3_wgrad<CIN, COUT><<<dim3(9, COUT / 16, chunks), 128, S::bytes, s>>>(X, dY, dW, N, H, Wd, chunks);
}

template <int CIN, int COUT>
int prep_t() {
  if (cudaFuncSetAttribute(jmgnet::k_conv3x3<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           jmgnet::ConvSmem<CIN, COUT>::bytes) != cudaSuccess)
    return 1;
  if (cudaFuncSetAttribute(jmgnet::k_conv3x3_wgrad<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           jmgnet::WgSmem<CIN, COUT>::bytes) != cudaSuccess)
    return 1;
  if (cudaFuncSetAttribute(jmgnet::k_conv3x3_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           jmgnet::TcConv<CIN, COUT>::smem) != cudaSuccess)
    return 1;
  return 0;
}

#define JMG_NET_SHAPES(X) X(16, 16) X(16, 32) X(32, 32) X(32, 64) X(64, 64) X(64, 32) X(32, 16)

int prepare_all() {
  int e = 0;
#define P_(a, b) e |= prep_t<a, b>();
  JMG_NET_SHAPES(P_)
#undef P_
  return e;
}

bool conv(int cin, int cout, const bf16* X, const bf16* W, const float* bias, const bf16* mask, bf16* Y, float* Y32,
          int N, int H, int Wd, int relu, int* fault, cudaStream_t s) {
#define C_(a, b)                                                      \
  if (cin == a && cout == b) {                                        \
    conv_t<a, b>(X, W, bias, mask, Y, Y32, N, H, Wd, relu, fault, s); \
    return true;                                                      \
  }
  JMG_NET_SHAPES(C_)
#undef C_
  return false;
}

bool wgrad(int cin, int cout, const bf16* X, const bf16* dY, float* dW, int N, int H, int Wd, cudaStream_t s) {
#define G_(a, b)                                  \
  if (cin == a && cout == b) {                    \
    wgrad_t<a, b>(X, dY, dW, N, H, Wd, s);        \
    return true;                                  \
  }
  JMG_NET_SHAPES(G_)
#undef G_
  return false;
}

// ---- inputs and outputs of the solver --------------------------------------------------

// pooled channels of one problem: tmp[(a * res + b) * 4 + c], block f x f of the padded
// grid starting at index 1 + f * a (y), 1 + f * b (x)
__global__ void k_net_pool(int m, int f, int res, const double* lam, double lam_s, const double* dxx, double dxx_s,
                           const double* dyy, double dyy_s, const double* rhs, float* tmp) {
  const int n = res * res;
  const int w = m + 3;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int a = t / res, b = t % res;
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int dy = 0; dy < f; ++dy)
      for (int dx = 0; dx < f; ++dx) {
        const size_t p = (size_t)(1 + f * a + dy) * w + (1 + f * b + dx);
        s0 += log(dxx ? dxx[p] : dxx_s);
        s1 += log(dyy ? dyy[p] : dyy_s);
        s2 += lam ? lam[p] : lam_s;
        s3 += rhs[p];
      }
    const double inv = 1.0 / (f * f);
    tmp[t * 4 + 0] = (float)(s0 * inv);
    tmp[t * 4 + 1] = (float)(s1 * inv);
    tmp[t * 4 + 2] = (float)(s2 * inv * 0.1);
    tmp[t * 4 + 3] = (float)(s3 * inv);
  }
}

// rms of the pooled rhs (one block, fixed order): rms[0]
__global__ void k_net_rms(const float* tmp, int n, float* rms) {
  __shared__ double part[1024];
  double s = 0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const double v = tmp[t * 4 + 3];
    s += v * v;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double r = sqrt(part[0] / n);
    rms[0] = (float)(r > 0 ? r : 1.0);
  }
}

// BF16 NHWC16 input: channels 0..3 from tmp (rhs divided by the rms), 4..15 zero
__global__ void k_net_pack(const float* tmp, const float* rms, int n, bf16* x) {
  const float ir = 1.f / rms[0];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    uint4 z[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    bf16* zb = reinterpret_cast<bf16*>(z);
    zb[0] = __float2bfloat16(tmp[t * 4 + 0]);
    zb[1] = __float2bfloat16(tmp[t * 4 + 1]);
    zb[2] = __float2bfloat16(tmp[t * 4 + 2]);
    zb[3] = __float2bfloat16(tmp[t * 4 + 3] * ir);
    uint4* o = reinterpret_cast<uint4*>(x + (size_t)t * 16);
    o[0] = z[0];
    o[1] = z[1];
  }
}

// phi0 on the padded grid from the network output y[res][res] (channel 0 of y32):
// phi0 = out_scale * rms * bilinear(y) on the interior (pixel centres at index
// 1 + f * a + (f - 1) / 2, clamped at the edges), zero on the frame
__global__ void k_net_out(const float* y32, const float* rms, float out_scale, int m, int f, int res, double* phi0) {
  const int w = m + 3;
  const int n = w * w;
  const double sc = (double)out_scale * (double)rms[0];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int j = t / w, i = t % w;
    double v = 0;
    if (i >= 2 && i <= m && j >= 2 && j <= m) {
      const double u = (i - 1 - 0.5 * (f - 1)) / f, q = (j - 1 - 0.5 * (f - 1)) / f;
      int b0 = (int)floor(u), a0 = (int)floor(q);
      double wu = u - b0, wq = q - a0;
      if (b0 < 0) { b0 = 0; wu = 0; }
      if (b0 > res - 2) { b0 = res - 2; wu = u - b0 > 1 ? 1 : u - b0; }
      if (a0 < 0) { a0 = 0; wq = 0; }
      if (a0 > res - 2) { a0 = res - 2; wq = q - a0 > 1 ? 1 : q - a0; }
      auto Y = [&](int a, int b) { return (double)y32[((size_t)a * res + b) * 16]; };
      const double top = (1 - wu) * Y(a0, b0) + wu * Y(a0, b0 + 1);
      const double bot = (1 - wu) * Y(a0 + 1, b0) + wu * Y(a0 + 1, b0 + 1);
      v = sc * ((1 - wq) * top + wq * bot);
    }
    phi0[t] = v;
  }
}

// Ritz scale of the guess g: beta = (g . rhs) / (g . L g) minimises the energy-norm
// error ||phi - beta g||_A for A = -L (SPD), L the level-0 operator built from the raw
// coefficients as the solver builds it (2D face averages, solver_2d.py:341-416).
// Partials per block: parts[2 b] = g . rhs, parts[2 b + 1] = g . L g (interior points).
constexpr int kRitzBlocks = 304;
__global__ void k_net_ritz_parts(const double* g, const double* rhs, int m, double idx2, double idy2, const double* lam,
                                 double lam_s, const double* dxx, double dxx_s, const double* dyy, double dyy_s,
                                 double* parts) {
  const int w = m + 3, n = (m - 1) * (m - 1);
  double a = 0.0, b = 0.0;
  auto Dx = [&](size_t p) { return dxx ? dxx[p] : dxx_s; };
  auto Dy = [&](size_t p) { return dyy ? dyy[p] : dyy_s; };
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 2 + t % (m - 1), j = 2 + t / (m - 1);
    const size_t p = (size_t)j * w + i;
    const double ex = 0.5 * (Dx(p) + Dx(p + 1)) * idx2, wx = 0.5 * (Dx(p - 1) + Dx(p)) * idx2;
    const double ny = 0.5 * (Dy(p) + Dy(p + w)) * idy2, sy = 0.5 * (Dy(p - w) + Dy(p)) * idy2;
    const double cc = ex + wx + ny + sy + (lam ? lam[p] : lam_s);
    const double lg = ex * g[p + 1] + wx * g[p - 1] + ny * g[p + w] + sy * g[p - w] - cc * g[p];
    a = fma(g[p], rhs[p], a);
    b = fma(g[p], lg, b);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  __shared__ double sa[32], sb[32];
  if ((threadIdx.x & 31) == 0) {
    sa[threadIdx.x >> 5] = a;
    sb[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0, tb = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      ta += sa[k];
      tb += sb[k];
    }
    parts[2 * blockIdx.x] = ta;
    parts[2 * blockIdx.x + 1] = tb;
  }
}

// g *= beta (beta from the partials, summed in a fixed order by every block)
__global__ void k_net_ritz_scale(double* g, int n, const double* parts) {
  __shared__ double beta;
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < kRitzBlocks; ++k) {
      a += parts[2 * k];
      b += parts[2 * k + 1];
    }
    beta = (b != 0.0 && a / b > 0.0) ? a / b : 0.0;
  }
  __syncthreads();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) g[t] *= beta;
}

// training target: block average of phi over the same f x f blocks as the inputs,
// divided by out_scale * rms
__global__ void k_net_target(const double* phi, const float* rms, float out_scale, int m, int f, int res,
                             float* target) {
  const int n = res * res, w = m + 3;
  const double sc = 1.0 / ((double)out_scale * (double)rms[0]);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int a = t / res, b = t % res;
    double s = 0;
    for (int dy = 0; dy < f; ++dy)
      for (int dx = 0; dx < f; ++dx) s += phi[(size_t)(1 + f * a + dy) * w + (1 + f * b + dx)];
    target[t] = (float)(s / (f * f) * sc);
  }
}

}  // namespace

struct JmgNet {
  int res = 0, max_batch = 0;
  long long step = 0;
  float* params = nullptr;  // FP32 master weights
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  bf16* wb = nullptr;       // BF16 weights per layer, forward layout
  bf16* wt = nullptr;       // BF16 weights per layer, transposed + flipped
  size_t wpos[kLayers];     // element offset of layer l in wb / wt
  // activations: a[l] (l < 11), pools p0..p2, up-adds u0..u2, y32; and their gradients
  bf16* act[kLayers];
  bf16* pool[3];
  bf16* up[3];
  bf16* gact[kLayers];
  bf16* gpool[3];
  bf16* gup[3];
  float* y32 = nullptr;
  bf16* gy = nullptr;
  bf16* x1 = nullptr;       // one packed input (guess path)
  float* tmp = nullptr;     // pooled input channels
  float* rms = nullptr;
  float* loss_scratch = nullptr;
  double* ritz_parts = nullptr;
  int* fault = nullptr;     // set by a tcgen05 convolution whose wait ran out
  std::vector<void*> allocs;

  template <typename T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T) < 256 ? 256 : n * sizeof(T)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return static_cast<T*>(p);
  }
  size_t pix(int lev, int batch) const {
    const size_t r = (size_t)(res >> lev);
    return r * r * batch;
  }
};

namespace {

int net_err(const char* msg) { return jmg::set_error_message(JMG_ERR_VALUE, msg); }

int cuda_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return JMG_OK;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return jmg::set_error_message(JMG_ERR_CUDA, buf);
}

void forward(JmgNet* n, const bf16* x, int B, cudaStream_t s) {
  const int R = n->res;
  auto L = [&](int l, const bf16* in, bf16* out, float* out32) {
    const LayerDesc& d = kNet[l];
    const int r = R >> d.lev;
    conv(d.cin, d.cout, in, n->wb + n->wpos[l], n->params + w_off(l) + w_elems(l), nullptr, out, out32, B, r, r,
         d.relu, n->fault, s);
  };
  auto pool = [&](const bf16* in, bf16* out, int lev, int C) {
    const int r = R >> lev;
    jmgnet::k_pool2<<<grid_for(n->pix(lev + 1, B) * C), 256, 0, s>>>(in, out, B, r, r, C);
  };
  auto upadd = [&](const bf16* coarse, const bf16* skip, bf16* out, int lev, int C) {
    const int r = R >> lev;
    jmgnet::k_up2_add<<<grid_for(n->pix(lev, B) * C), 256, 0, s>>>(coarse, skip, out, B, r, r, C);
  };
  L(0, x, n->act[0], nullptr);
  L(1, n->act[0], n->act[1], nullptr);
  pool(n->act[1], n->pool[0], 0, 16);
  L(2, n->pool[0], n->act[2], nullptr);
  L(3, n->act[2], n->act[3], nullptr);
  pool(n->act[3], n->pool[1], 1, 32);
  L(4, n->pool[1], n->act[4], nullptr);
  L(5, n->act[4], n->act[5], nullptr);
  pool(n->act[5], n->pool[2], 2, 64);
  L(6, n->pool[2], n->act[6], nullptr);
  L(7, n->act[6], n->act[7], nullptr);
  upadd(n->act[7], n->act[5], n->up[2], 2, 64);
  L(8, n->up[2], n->act[8], nullptr);
  upadd(n->act[8], n->act[3], n->up[1], 1, 32);
  L(9, n->up[1], n->act[9], nullptr);
  upadd(n->act[9], n->act[1], n->up[0], 0, 16);
  L(10, n->up[0], n->act[10], nullptr);
  L(11, n->act[10], nullptr, n->y32);
}

// gradients of the mean squared error into n->grads (zeroed here), loss added to *loss
void backward(JmgNet* n, const bf16* x, const float* target, int B, float* loss, cudaStream_t s) {
  const int R = n->res;
  cudaMemsetAsync(n->grads, 0, num_params() * sizeof(float), s);
  jmgnet::k_mse<<<grid_for(n->pix(0, B)), 256, 0, s>>>(n->y32, target, n->gy, loss, n->pix(0, B));
  // one layer: weight and bias gradients from (input, output gradient); the input
  // gradient (through the ReLU of the layer below when `mask` is set) into `gin`
  auto back = [&](int l, const bf16* in, const bf16* gout, const bf16* mask, bf16* gin) {
    const LayerDesc& d = kNet[l];
    const int r = R >> d.lev;
    float* gw = n->grads + w_off(l);
    wgrad(d.cin, d.cout, in, gout, gw, B, r, r, s);
    const size_t np = n->pix(d.lev, B);
    jmgnet::k_bias_grad<<<dim3(grid_for(np) > 64 ? 64 : grid_for(np), d.cout), 256, 0, s>>>(gout, gw + w_elems(l), np,
                                                                                             d.cout);
    if (gin)
      conv(d.cout, d.cin, gout, n->wt + n->wpos[l], nullptr, mask, gin, nullptr, B, r, r, 0, n->fault, s);
  };
  auto upbwd = [&](const bf16* gu, const bf16* mask, bf16* gc, int lev, int C) {
    const int r = R >> lev;
    jmgnet::k_up2_bwd<<<grid_for(n->pix(lev + 1, B) * C), 256, 0, s>>>(gu, mask, gc, B, r, r, C);
  };
  auto poolbwd = [&](const bf16* gp, const bf16* add, const bf16* mask, bf16* gx, int lev, int C) {
    const int r = R >> lev;
    jmgnet::k_pool2_bwd<<<grid_for(n->pix(lev, B) * C), 256, 0, s>>>(gp, add, mask, gx, B, r, r, C);
  };
  back(11, n->act[10], n->gy, n->act[10], n->gact[10]);
  back(10, n->up[0], n->gact[10], nullptr, n->gup[0]);
  upbwd(n->gup[0], n->act[9], n->gact[9], 0, 16);
  back(9, n->up[1], n->gact[9], nullptr, n->gup[1]);
  upbwd(n->gup[1], n->act[8], n->gact[8], 1, 32);
  back(8, n->up[2], n->gact[8], nullptr, n->gup[2]);
  upbwd(n->gup[2], n->act[7], n->gact[7], 2, 64);
  back(7, n->act[6], n->gact[7], n->act[6], n->gact[6]);
  back(6, n->pool[2], n->gact[6], nullptr, n->gpool[2]);
  poolbwd(n->gpool[2], n->gup[2], n->act[5], n->gact[5], 2, 64);
  back(5, n->act[4], n->gact[5], n->act[4], n->gact[4]);
  back(4, n->pool[1], n->gact[4], nullptr, n->gpool[1]);
  poolbwd(n->gpool[1], n->gup[1], n->act[3], n->gact[3], 1, 32);
  back(3, n->act[2], n->gact[3], n->act[2], n->gact[2]);
  back(2, n->pool[0], n->gact[2], nullptr, n->gpool[0]);
  poolbwd(n->gpool[0], n->gup[0], n->act[1], n->gact[1], 0, 16);
  back(1, n->act[0], n->gact[1], n->act[0], n->gact[0]);
  back(0, x, n->gact[0], nullptr, nullptr);
}

void pack_all(JmgNet* n, cudaStream_t s) {
  for (int l = 0; l < kLayers; ++l)
    jmgnet::k_pack_weights<<<grid_for(w_elems(l)), 256, 0, s>>>(n->params + w_off(l), n->wb + n->wpos[l],
                                                                n->wt + n->wpos[l], kNet[l].cout, kNet[l].cin);
}

int check_batch(const JmgNet* n, int batch) {
  if (!n) return net_err("net must not be NULL");
  if (batch < 1 || batch > n->max_batch) return net_err("batch must be in [1, max_batch]");
  return JMG_OK;
}

// pooled, normalised inputs of one 2D problem into x (BF16 NHWC16), rms into n->rms
int inputs_2d(JmgNet* n, const JmgGrid* g, const JmgCoeffs* c, const double* rhs, bf16* x, cudaStream_t s) {
  if (!g || !c || !rhs || !x) return net_err("grid, coeffs, rhs and x must not be NULL");
  if (g->ndim != 2 || g->m[0] != g->m[1]) return net_err("the learned guess takes square 2D grids");
  const int m = g->m[0], R = n->res;
  if (m < R || m % R) return net_err("grid resolution must be a multiple of the network resolution");
  const int f = m / R;
  k_net_pool<<<grid_for((size_t)R * R), 256, 0, s>>>(m, f, R, c->lam, c->lam_scalar, c->D[0], c->D_scalar[0], c->D[1],
                                                     c->D_scalar[1], rhs, n->tmp);
  k_net_rms<<<1, 1024, 0, s>>>(n->tmp, R * R, n->rms);
  k_net_pack<<<grid_for((size_t)R * R), 256, 0, s>>>(n->tmp, n->rms, R * R, x);
  return JMG_OK;
}

}  // namespace

extern "C" {

int64_t jmg_net_num_params(void) { return (int64_t)num_params(); }

int jmg_net_create(JmgNet** out, int res, int max_batch) {
  if (!out) return net_err("out must not be NULL");
  *out = nullptr;
  if (res < 128 || res % 128) return net_err("network resolution must be a positive multiple of 128");
  if (max_batch < 1) return net_err("max_batch must be >= 1");
  if (prepare_all()) return cuda_check("cannot set the shared-memory size of the convolution kernels");
  JmgNet* n = new JmgNet;
  n->res = res;
  n->max_batch = max_batch;
  const size_t P = num_params();
  size_t wtot = 0;
  for (int l = 0; l < kLayers; ++l) {
    n->wpos[l] = wtot;
    wtot += w_elems(l);
  }
  bool ok = (n->params = n->alloc<float>(P)) && (n->grads = n->alloc<float>(P)) && (n->adam_m = n->alloc<float>(P)) &&
            (n->adam_v = n->alloc<float>(P)) && (n->wb = n->alloc<bf16>(wtot)) && (n->wt = n->alloc<bf16>(wtot));
  const int B = max_batch;
  for (int l = 0; ok && l < kLayers; ++l) {
    n->act[l] = n->gact[l] = nullptr;
    if (l == 11) continue;
    ok = (n->act[l] = n->alloc<bf16>(n->pix(kNet[l].lev, B) * kNet[l].cout)) &&
         (n->gact[l] = n->alloc<bf16>(n->pix(kNet[l].lev, B) * kNet[l].cout));
  }
  const int pc[3] = {16, 32, 64};
  for (int k = 0; ok && k < 3; ++k) {
    ok = (n->pool[k] = n->alloc<bf16>(n->pix(k + 1, B) * pc[k])) &&
         (n->gpool[k] = n->alloc<bf16>(n->pix(k + 1, B) * pc[k])) &&
         (n->up[k] = n->alloc<bf16>(n->pix(k, B) * pc[k])) && (n->gup[k] = n->alloc<bf16>(n->pix(k, B) * pc[k]));
  }
  ok = ok && (n->y32 = n->alloc<float>(n->pix(0, B) * 16)) && (n->gy = n->alloc<bf16>(n->pix(0, B) * 16)) &&
       (n->x1 = n->alloc<bf16>(n->pix(0, 1) * 16)) && (n->tmp = n->alloc<float>(n->pix(0, 1) * 4)) &&
       (n->rms = n->alloc<float>(1)) && (n->loss_scratch = n->alloc<float>(1)) &&
       (n->ritz_parts = n->alloc<double>(2 * kRitzBlocks)) && (n->fault = n->alloc<int>(1));
  if (!ok) {
    jmg_net_destroy(n);
    return jmg::set_error_message(JMG_ERR_CUDA, "cudaMalloc failed while creating the network");
  }
  if (cudaMemset(n->fault, 0, sizeof(int)) != cudaSuccess || cudaMemset(n->params, 0, P * sizeof(float)) != cudaSuccess || cudaMemset(n->adam_m, 0, P * 4) != cudaSuccess ||
      cudaMemset(n->adam_v, 0, P * 4) != cudaSuccess) {
    jmg_net_destroy(n);
    return cuda_check("cudaMemset");
  }
  *out = n;
  return JMG_OK;
}

void jmg_net_destroy(JmgNet* n) {
  if (!n) return;
  for (void* p : n->allocs) cudaFree(p);
  delete n;
}

int jmg_net_set_params(JmgNet* n, const float* params, jmg_stream_t stream) {
  if (!n || !params) return net_err("net and params must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemcpyAsync(n->params, params, num_params() * sizeof(float), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(n->adam_m, 0, num_params() * sizeof(float), s);
  cudaMemsetAsync(n->adam_v, 0, num_params() * sizeof(float), s);
  n->step = 0;
  pack_all(n, s);
  return cuda_check("jmg_net_set_params");
}

int jmg_net_get_params(JmgNet* n, float* params, jmg_stream_t stream) {
  if (!n || !params) return net_err("net and params must not be NULL");
  cudaMemcpyAsync(params, n->params, num_params() * sizeof(float), cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  return cuda_check("jmg_net_get_params");
}

int jmg_net_forward(JmgNet* n, const void* x, int batch, float* y, jmg_stream_t stream) {
  int rc = check_batch(n, batch);
  if (rc) return rc;
  if (!x || !y) return net_err("x and y must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  forward(n, static_cast<const bf16*>(x), batch, s);
  jmgnet::k_take_channel0<<<grid_for(n->pix(0, batch)), 256, 0, s>>>(n->y32, y, n->pix(0, batch));
  return cuda_check("jmg_net_forward");
}

int jmg_net_loss_grad(JmgNet* n, const void* x, const float* target, int batch, float* loss, float* grads,
                      jmg_stream_t stream) {
  int rc = check_batch(n, batch);
  if (rc) return rc;
  if (!x || !target || !loss) return net_err("x, target and loss must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  forward(n, static_cast<const bf16*>(x), batch, s);
  cudaMemsetAsync(loss, 0, sizeof(float), s);
  backward(n, static_cast<const bf16*>(x), target, batch, loss, s);
  if (grads) cudaMemcpyAsync(grads, n->grads, num_params() * sizeof(float), cudaMemcpyDeviceToDevice, s);
  return cuda_check("jmg_net_loss_grad");
}

int jmg_net_train_step(JmgNet* n, const void* x, const float* target, int batch, float lr, float* loss,
                       jmg_stream_t stream) {
  int rc = check_batch(n, batch);
  if (rc) return rc;
  if (!x || !target) return net_err("x and target must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  float* l = loss ? loss : n->loss_scratch;
  forward(n, static_cast<const bf16*>(x), batch, s);
  if (!loss) cudaMemsetAsync(l, 0, sizeof(float), s);
  backward(n, static_cast<const bf16*>(x), target, batch, l, s);
  ++n->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
  jmgnet::k_adam<<<grid_for(num_params()), 256, 0, s>>>(n->params, n->grads, n->adam_m, n->adam_v, num_params(), lr,
                                                        b1, b2, 1e-8f, c1, c2);
  pack_all(n, s);
  return cuda_check("jmg_net_train_step");
}

int jmg_net_inputs_2d(JmgNet* n, const JmgGrid* grid, const JmgCoeffs* coeffs, const double* rhs, void* x,
                      float* rms_out, jmg_stream_t stream) {
  if (!n) return net_err("net must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = inputs_2d(n, grid, coeffs, rhs, static_cast<bf16*>(x), s);
  if (rc) return rc;
  if (rms_out) cudaMemcpyAsync(rms_out, n->rms, sizeof(float), cudaMemcpyDeviceToDevice, s);
  return cuda_check("jmg_net_inputs_2d");
}

int jmg_net_target_2d(JmgNet* n, const JmgGrid* grid, const double* phi, const float* rms, float out_scale,
                      float* target, jmg_stream_t stream) {
  if (!n || !grid || !phi || !rms || !target) return net_err("net, grid, phi, rms and target must not be NULL");
  if (grid->ndim != 2 || grid->m[0] != grid->m[1]) return net_err("the learned guess takes square 2D grids");
  const int m = grid->m[0], R = n->res;
  if (m < R || m % R) return net_err("grid resolution must be a multiple of the network resolution");
  k_net_target<<<grid_for((size_t)R * R), 256, 0, (cudaStream_t)stream>>>(phi, rms, out_scale, m, m / R, R, target);
  return cuda_check("jmg_net_target_2d");
}

int jmg_net_guess_2d(JmgNet* n, const JmgGrid* grid, const JmgCoeffs* coeffs, const double* rhs, float out_scale,
                     double* phi0, jmg_stream_t stream) {
  if (!n || !phi0) return net_err("net and phi0 must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = inputs_2d(n, grid, coeffs, rhs, n->x1, s);
  if (rc) return rc;
  forward(n, n->x1, 1, s);
  const int m = grid->m[0], R = n->res;
  const int np = (m + 3) * (m + 3);
  k_net_out<<<grid_for((size_t)np), 256, 0, s>>>(n->y32, n->rms, out_scale, m, m / R, R, phi0);
  k_net_ritz_parts<<<kRitzBlocks, 256, 0, s>>>(phi0, rhs, m, grid->idel[0] * grid->idel[0],
                                               grid->idel[1] * grid->idel[1], coeffs->lam, coeffs->lam_scalar,
                                               coeffs->D[0], coeffs->D_scalar[0], coeffs->D[1], coeffs->D_scalar[1],
                                               n->ritz_parts);
  k_net_ritz_scale<<<grid_for((size_t)np), 256, 0, s>>>(phi0, np, n->ritz_parts);
  return cuda_check("jmg_net_guess_2d");
}

}  // extern "C"
