// mg_aux.cu — layout copies, reductions and the device-side loop control.
//
// The dynamic loop of the reference (lax.while_loop over `dist > epsilon and count <
// max_iters_outer`, solver_2d.py:465-477) runs on the device as a conditional WHILE
// node of a CUDA graph: k_loop_step evaluates the predicate after every cycle and sets
// the node's condition with cudaGraphSetConditional, so no host round trip happens
// between cycles. The distance (solver_2d.py:481-494) is max |phi_old - phi| over the
// whole padded array, reduced as ordered bit patterns so that NaN propagates.
// Sums of squares are reduced in a fixed order (fixed grid, per-block partials, one warp
// for the final sum), so the residual norm is bitwise reproducible from run to run.
#include <algorithm>

#include "mg_kernels.h"

namespace jmg {

static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// ------------------------------------------------------------------------------------
// dense <-> pitched copies
// ------------------------------------------------------------------------------------

__global__ void k_copy_in(Box b, const double* __restrict__ src, double* __restrict__ dst, int zero_frame) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  double v = src[((long long)K * b.ny + J) * b.nx + I];
  if (zero_frame) {
    const bool fr = I < 2 || I >= b.nx - 2 || J < 2 || J >= b.ny - 2 || (b.nz > 1 && (K < 2 || K >= b.nz - 2));
    if (fr) v = 0.0;
  }
  dst[(long long)K * b.S + (long long)J * b.P + I] = v;
}

__global__ void k_copy_out(Box b, const double* __restrict__ src, double* __restrict__ dst) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  dst[((long long)K * b.ny + J) * b.nx + I] = src[(long long)K * b.S + (long long)J * b.P + I];
}

void launch_copy_in(const Box& b, const double* src, double* dst, int zero_frame, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz);
  k_copy_in<<<g, blk, 0, s>>>(b, src, dst, zero_frame);
}

void launch_copy_out(const Box& b, const double* src, double* dst, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz);
  k_copy_out<<<g, blk, 0, s>>>(b, src, dst);
}

void launch_copy_coeff(const Box& b, const double* src, double* dst, cudaStream_t s) { launch_copy_out(b, src, dst, s); }

// do_BCs on a dense array of any padded shape (rim 1, zero values)
__global__ void k_do_bcs_dense(int nx, int ny, int nz, double* a) {
  const long long n = (long long)nx * ny * nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(t % nx);
    const int J = (int)((t / nx) % ny);
    const int K = (int)(t / ((long long)nx * ny));
    const bool fr = I < 2 || I >= nx - 2 || J < 2 || J >= ny - 2 || (nz > 1 && (K < 2 || K >= nz - 2));
    if (fr) a[t] = 0.0;
  }
}

void launch_do_bcs_dense(int dim, const int32_t* shape, double* arr, cudaStream_t s) {
  const int nz = dim == 3 ? shape[0] : 1, ny = shape[dim - 2], nx = shape[dim - 1];
  const long long n = (long long)nx * ny * nz;
  const unsigned g = (unsigned)std::min<long long>(cdiv(n, 256), 4096);
  k_do_bcs_dense<<<g, 256, 0, s>>>(nx, ny, nz, arr);
}

// ------------------------------------------------------------------------------------
// distance + snapshot
// ------------------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

__global__ void k_distance_snapshot(Box b, double* __restrict__ old_phi, const double* __restrict__ phi,
                                    LoopState* st) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  unsigned long long m = 0;
  if (I < b.nx && J < b.ny) {
    const long long p = (long long)K * b.S + (long long)J * b.P + I;
    const double n = phi[p];
    m = abs_bits(old_phi[p] - n);
    old_phi[p] = n;
  }
  m = warp_max_u64(m);
  __shared__ unsigned long long sm[32];
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31, wid = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
  if (lane == 0) sm[wid] = m;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x * blockDim.y) >> 5;
    m = lane < nw ? sm[lane] : 0;
    m = warp_max_u64(m);
    if (lane == 0 && m) atomicMax(&st->dist_bits, m);
  }
}

void launch_distance_snapshot(const Box& b, double* old_phi, const double* phi, LoopState* st, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz);
  launch_k(k_distance_snapshot, g, blk, 0, s, b, old_phi, phi, st);
}

// ------------------------------------------------------------------------------------
// residual norms (deterministic)
// ------------------------------------------------------------------------------------

// 304 blocks (2 per SM) up to 4096 interior rows, 1216 (8 per SM) above: fixed per
// problem size, so the reduction order, and the result, is reproducible
inline int res_blocks(const Box& b) { return (b.ny - 3) * (b.nz > 1 ? b.nz - 3 : 1) > 4096 ? 1216 : 304; }
constexpr int kResThreads = 256;

int residual_num_parts(int, const Box& b) { return res_blocks(b); }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sm[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sm[wid] = v;
  __syncthreads();
  v = 0.0;
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
    v = warp_sum(v);
  }
  return v;
}

// sum over interior points of d^2, d = rhs - L_h phi (phi == nullptr: d = rhs); with r32,
// d is also stored as FP32 (the right-hand side of the next refinement step)
// Interior rows (2D: j; 3D: (k, j)) are dealt to the blocks round-robin and the threads
// of a block walk each row: one 32-bit division per row, fixed reduction order.
template <typename T, int DIM>
__global__ void k_residual_partials(Lvl<T> a, const T* phi, double* parts, float* r32) {
  pdl_enter();
  const int ny = a.my - 1, nz = DIM == 3 ? a.mz - 1 : 1;
  const int nrows = ny * nz;
  double acc = 0.0;
  for (int r = blockIdx.x; r < nrows; r += gridDim.x)
  for (int i = 2 + threadIdx.x; i <= a.mx; i += blockDim.x) {
    const int k = DIM == 3 ? 2 + r / ny : 0;
    const int j = 2 + (DIM == 3 ? r % ny : r);
    const long long p = DIM == 2 ? (long long)j * a.P + i : (long long)k * a.S + (long long)j * a.P + i;
    double d;
    if (phi == nullptr) d = (double)a.rhs[p];
    else if (DIM == 2) d = (double)defect_point2d<T>(a, phi, p);
    else d = (double)defect_point3d<T>(phi, a.rhs, a.wx, a.wy, a.wz, a.acc, p, a.P, a.S);
    if (r32) r32[p] = (float)d;
    acc = fma(d, d, acc);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) parts[blockIdx.x] = acc;
}

template <typename T>
void launch_residual_partials(int dim, const Lvl<T>& a, const T* phi_or_null, double* parts, int nparts, cudaStream_t s,
                              float* r32) {
  if (dim == 2)
    launch_k(k_residual_partials<T, 2>, dim3(nparts), dim3(kResThreads), 0, s, a, phi_or_null, parts, r32);
  else
    launch_k(k_residual_partials<T, 3>, dim3(nparts), dim3(kResThreads), 0, s, a, phi_or_null, parts, r32);
}
template void launch_residual_partials<double>(int, const Lvl<double>&, const double*, double*, int, cudaStream_t,
                                               float*);

__device__ double reduce_parts_warp(const double* parts, int n) {
  // called by one full warp; fixed assignment of parts to lanes, fixed shuffle tree
  double v = 0.0;
#pragma unroll 8
  for (int t = threadIdx.x; t < n; t += 32) v += parts[t];  // unrolled: loads in flight together
  return warp_sum(v);
}

// ------------------------------------------------------------------------------------
// loop control
// ------------------------------------------------------------------------------------

// mode: 0 = distance (reference dynamic loop), 1 = relative residual, 2 = fixed count
__global__ void k_loop_init(LoopState* st, const double* parts, int nparts, int mode, double rtol,
                            long long max_iters, unsigned long long handle) {
  double r = 0.0;
  if (mode == 1) r = sqrt(reduce_parts_warp(parts, nparts));
  if (threadIdx.x != 0) return;
  st->count = 0;
  st->dist_bits = 0;
  st->fault = 0;
  st->bar_count = 0;
  int go = max_iters > 0;
  if (mode == 1) {
    st->res_norm = r;
    st->rel_res = r / st->rhs_norm;
    go = go && (st->rel_res > rtol);
  }
  st->go = go;
  if (handle) cudaGraphSetConditional((cudaGraphConditionalHandle)handle, go ? 1u : 0u);
}

__global__ void k_loop_step(LoopState* st, const double* parts, int nparts, int mode, double eps, double rtol,
                            long long max_iters, unsigned long long handle) {
  pdl_enter();
  double r = 0.0;
  if (mode == 1) r = sqrt(reduce_parts_warp(parts, nparts));
  if (threadIdx.x != 0) return;
  const long long c = st->count + 1;
  st->count = c;
  int go = c < max_iters;
  if (mode == 0) {
    const double dist = __longlong_as_double((long long)st->dist_bits);
    go = go && (dist > eps);  // NaN distance ends the loop, as in the reference
    st->dist_bits = 0;
  } else if (mode == 1) {
    st->res_norm = r;
    st->rel_res = r / st->rhs_norm;
    go = go && (st->rel_res > rtol);
  }
  if (st->fault) go = 0;  // a bounded wait ran out: the iterate is void, stop
  st->go = go;
  if (handle) cudaGraphSetConditional((cudaGraphConditionalHandle)handle, go ? 1u : 0u);
}

__global__ void k_rhs_norm(LoopState* st, const double* parts, int nparts) {
  const double r = sqrt(reduce_parts_warp(parts, nparts));
  if (threadIdx.x == 0) st->rhs_norm = r;
}

__global__ void k_rel_residual_out(const LoopState* st, const double* parts, int nparts, double* out) {
  const double r = sqrt(reduce_parts_warp(parts, nparts));
  if (threadIdx.x == 0) *out = r / st->rhs_norm;
}

__global__ void k_count_out(const LoopState* st, long long* out) { *out = st->count; }

void launch_loop_init(LoopState* st, const double* parts, int nparts, int mode, double rtol, long long max_iters,
                      unsigned long long h, cudaStream_t s) {
  k_loop_init<<<1, 32, 0, s>>>(st, parts, nparts, mode, rtol, max_iters, h);
}
void launch_loop_step(LoopState* st, const double* parts, int nparts, int mode, double eps, double rtol,
                      long long max_iters, unsigned long long h, cudaStream_t s) {
  launch_k(k_loop_step, dim3(1), dim3(32), 0, s, st, parts, nparts, mode, eps, rtol, max_iters, h);
}
void launch_rhs_norm(LoopState* st, const double* parts, int nparts, cudaStream_t s) {
  k_rhs_norm<<<1, 32, 0, s>>>(st, parts, nparts);
}
void launch_rel_residual_out(const LoopState* st, const double* parts, int nparts, double* out, cudaStream_t s) {
  k_rel_residual_out<<<1, 32, 0, s>>>(st, parts, nparts, out);
}
void launch_count_out(const LoopState* st, long long* out, cudaStream_t s) { k_count_out<<<1, 1, 0, s>>>(st, out); }

// ------------------------------------------------------------------------------------
// dense defect field (operator entry point)
// ------------------------------------------------------------------------------------

template <int DIM>
__global__ void k_dense_residual(Lvl<double> a, Box b, double* d) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  double v = 0.0;
  const bool in = I >= 2 && I <= a.mx && J >= 2 && J <= a.my && (DIM == 2 || (K >= 2 && K <= a.mz));
  if (in) {
    const long long p = (long long)K * a.S + (long long)J * a.P + I;
    v = DIM == 2 ? defect_point2d<double>(a, a.phi, p)
                 : defect_point3d<double>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.acc, p, a.P, a.S);
  }
  d[((long long)K * b.ny + J) * b.nx + I] = v;
}

void launch_dense_residual(int dim, const Lvl<double>& a, const Box& b, double* d, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz);
  if (dim == 2) k_dense_residual<2><<<g, blk, 0, s>>>(a, b, d);
  else k_dense_residual<3><<<g, blk, 0, s>>>(a, b, d);
}

// ------------------------------------------------------------------------------------
// mixed precision: FP64 residual -> FP32, FP64 update from FP32 correction
// ------------------------------------------------------------------------------------

template <int DIM>
__global__ void k_residual_to_f32(Lvl<double> a, float* r32) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I > a.mx + 2 || J > a.my + 2) return;
  const long long p = (long long)K * a.S + (long long)J * a.P + I;
  float v = 0.f;
  const bool in = I >= 2 && I <= a.mx && J >= 2 && J <= a.my && (DIM == 2 || (K >= 2 && K <= a.mz));
  if (in)
    v = (float)(DIM == 2 ? defect_point2d<double>(a, a.phi, p)
                         : defect_point3d<double>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.acc, p, a.P, a.S));
  r32[p] = v;
}

void launch_residual_to_f32(int dim, const Lvl<double>& a, float* r32, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(a.mx + 3, 32), cdiv(a.my + 3, 8), dim == 3 ? a.mz + 3 : 1);
  if (dim == 2) k_residual_to_f32<2><<<g, blk, 0, s>>>(a, r32);
  else k_residual_to_f32<3><<<g, blk, 0, s>>>(a, r32);
}

template <int DIM>
__global__ void k_add_correction(Lvl<double> a, const float* e32) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > a.mx || j > a.my) return;
  const long long p = DIM == 2 ? (long long)j * a.P + i : (long long)k * a.S + (long long)j * a.P + i;
  a.phi[p] += (double)e32[p];
}

void launch_add_correction(int dim, const Lvl<double>& a, const float* e32, cudaStream_t s) {
  dim3 blk(64, 4, 1), g(cdiv(a.mx - 1, 64), cdiv(a.my - 1, 4), dim == 3 ? a.mz - 1 : 1);
  if (dim == 2) launch_k(k_add_correction<2>, g, blk, 0, s, a, e32);
  else launch_k(k_add_correction<3>, g, blk, 0, s, a, e32);
}

__global__ void k_convert_f32(Box b, const double* src, float* dst) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  const long long p = (long long)K * b.S + (long long)J * b.P + I;
  dst[p] = src ? (float)src[p] : 0.f;
}

void launch_zero_f32(const Box& b, float* x, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz);
  k_convert_f32<<<g, blk, 0, s>>>(b, nullptr, x);
}

void launch_convert_f32(const Box& b, const double* src, float* dst, cudaStream_t s) {
  dim3 blk(32, 8, 1), g(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz);
  k_convert_f32<<<g, blk, 0, s>>>(b, src, dst);
}

}  // namespace jmg
