// mg_krylov.cu — flexible conjugate gradients around the multigrid cycle (outer = FCG).
//
// The reference iterates the cycle as a stationary method: phi <- phi + M(rhs - L phi).
// With JmgConfig.outer = JMG_OUTER_FCG the same cycle M (FP64, or FP32 inside FP64
// refinement) preconditions FCG(1), the flexible CG of Notay (SIAM J. Sci. Comput. 22,
// 2000) truncated to one previous direction, which tolerates a preconditioner that is
// neither symmetric nor fixed (a red-black V-cycle, FP32 rounding). With A = -L (SPD for
// D > 0, lambda >= 0) and rho = rhs - L x:
//   z = M(rho);  beta = (z . q) / (d . q);  d <- z - beta d;  q <- L z - beta q  (= L d)
//   alpha = (d . rho) / (d . q);  x <- x + alpha d;  rho <- rho - alpha q
// All vectors and dot products are FP64; the dot products are reduced in a fixed order
// (kBlocks per-block partials, summed by every consumer block in the same order), so a
// solve is bitwise reproducible. The stopping test reads ||rho||, the recurrence
// residual; it tracks the true residual to FP64 rounding over the few dozen steps a solve
// takes (checked against jmg_rel_residual in the tests).
#include <cstdlib>

#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

// Block count of the FCG kernels: 304 (2 per SM) for up to 4096 interior rows, 608 (4
// per SM) above (3D 256^3 headline: 104.2 ms against 106.3 with 1216 and 119 with 304;
// 2D 1024^2: 304 beats 608 and 1216). It depends on the problem size only, so for a
// given problem the reduction order is fixed and solves are bitwise reproducible.
constexpr int kBlocks = 1216;  // the most blocks (partials) any FCG kernel uses
inline int fcg_blocks(int rows) {
  // JMG_FCG_BLOCKS (152 .. 1216) overrides the choice for tuning runs
  static const int forced = [] {
    const char* e = getenv("JMG_FCG_BLOCKS");
    const int v = e ? atoi(e) : 0;
    return v >= 152 && v <= 1216 ? v : 0;
  }();
  if (forced) return forced;
  return rows > 4096 ? 608 : 304;
}
constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sums of two values over the block; valid in thread 0
__device__ __forceinline__ void block_sum2(double& a, double& b) {
  __shared__ double sa[32], sb[32];
  a = warp_sum(a);
  b = warp_sum(b);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sa[wid] = a;
    sb[wid] = b;
  }
  __syncthreads();
  if (wid == 0) {
    a = lane < (int)(blockDim.x >> 5) ? sa[lane] : 0.0;
    b = lane < (int)(blockDim.x >> 5) ? sb[lane] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
  }
}

// the two totals of a [kBlocks][2] partial array, in a fixed order, in every thread
__device__ __forceinline__ void totals2(const double* parts, double* t0, double* t1) {
  __shared__ double s[2];
  if (threadIdx.x < 32) {
    double a = 0.0, b = 0.0;
    // unrolled so that a lane's loads are in flight together (the sum order is unchanged)
#pragma unroll 8
    for (int t = threadIdx.x; t < (int)gridDim.x; t += 32) {
      a += parts[2 * t];
      b += parts[2 * t + 1];
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if (threadIdx.x == 0) {
      s[0] = a;
      s[1] = b;
    }
  }
  __syncthreads();
  *t0 = s[0];
  *t1 = s[1];
}

// Interior rows (2D: j; 3D: (k, j)) are dealt to the kBlocks blocks round-robin, and the
// threads of a block walk each row in x: one 32-bit division per row instead of 64-bit
// index arithmetic per point. The reduction order stays fixed.
template <int DIM>
__device__ __forceinline__ int nrows(const Lvl<double>& a) {
  return (a.my - 1) * (DIM == 3 ? a.mz - 1 : 1);
}
template <int DIM>
__device__ __forceinline__ long long row_base(const Lvl<double>& a, int r) {
  const int k = DIM == 3 ? 2 + r / (a.my - 1) : 0;
  const int j = 2 + (DIM == 3 ? r % (a.my - 1) : r);
  return DIM == 2 ? (long long)j * a.P : (long long)k * a.S + (long long)j * a.P;
}
#define JMG_FOR_POINTS(a, p)                                                          \
  for (int r_ = blockIdx.x; r_ < nrows<DIM>(a); r_ += gridDim.x)                      \
    for (long long base_ = row_base<DIM>(a, r_), i_ = 2 + threadIdx.x; i_ <= (a).mx; \
         i_ += kThreads)                                                              \
      if (const long long p = base_ + i_; true)

// L z at p (FP64 arithmetic on z's values): -(A_cc z - sum of couplings * neighbours),
// in the order of the defect (mg_common.cuh: defect_point2d/3d)
template <int DIM, typename TZ>
__device__ __forceinline__ double apply_L(const Lvl<double>& a, const TZ* z, long long p) {
  double t = a.acc[p] * (double)z[p];
  t = fma(-a.wx[p - 1], (double)z[p - 1], t);
  t = fma(-a.wx[p], (double)z[p + 1], t);
  t = fma(-a.wy[p - a.P], (double)z[p - a.P], t);
  t = fma(-a.wy[p], (double)z[p + a.P], t);
  if (DIM == 3) {
    t = fma(-a.wz[p - a.S], (double)z[p - a.S], t);
    t = fma(-a.wz[p], (double)z[p + a.S], t);
  }
  if (DIM == 2 && a.xll) {  // 9-point stencil (D_xy): the off-diagonal couplings
    const int P = a.P;
    double o = a.xll[p] * (double)z[p - P - 1];
    o = fma(a.xrl[p], (double)z[p - P + 1], o);
    o = fma(a.xlr[p], (double)z[p + P - 1], o);
    o = fma(a.xrr[p], (double)z[p + P + 1], o);
    t = t - o;
  }
  return -t;
}

// The streaming FCG kernels walk rows in groups of consecutive rows: each thread takes the same x in every row of a group and issues the group's loads
// together, so that a thread has several rows' loads in flight instead of one point's.
// (A 3D row of 255 points is one point per thread; with one row at a time the kernels
// were latency-bound at a third to a half of the DRAM bandwidth.) The order of every
// sum is still fixed by the problem size alone.
// Group sizes: 4 rows for the streaming kernels (dots, x update); the stencil kernels
// (direction, residual) take two rows in 2D and one in 3D, where the loads of one row
// already fill the registers (two rows per group: 80 registers, three blocks per SM,
// and a direction step of 322 instead of 186 us at 3D 256^3).
template <int DIM>
constexpr int kGroup = 4;
template <int DIM>
constexpr int kGroupStencil = DIM == 2 ? 2 : 1;

// rows of group g: their bases (0 where the row does not exist)
template <int DIM, int G>
__device__ __forceinline__ int group_rows(const Lvl<double>& a, int g, int nr, long long* base) {
  int n = 0;
#pragma unroll
  for (int u = 0; u < G; ++u) {
    const int r = g * G + u;
    base[u] = r < nr ? row_base<DIM>(a, r) : 0;
    n += r < nr;
  }
  return n;
}

#define JMG_FOR_GROUPS(a, G)                                                                 \
  for (int g_ = blockIdx.x, nr_ = nrows<DIM>(a); g_ * (G) < nr_; g_ += gridDim.x)           \
    for (long long base_[G], n_ = group_rows<DIM, G>(a, g_, nr_, base_), i_ = 2 + threadIdx.x; \
         i_ <= (a).mx; i_ += kThreads)

// rho = rhs - L x, d = q = 0, r32 = float(rho); partials of rho . rho
template <int DIM>
__global__ void __launch_bounds__(kThreads) k_fcg_init(Lvl<double> a, double* rho, double* d, double* q, float* r32,
                                                      double* parts) {
  pdl_enter();
  double s = 0.0, unused = 0.0;
  JMG_FOR_POINTS(a, p) {
    const double r = DIM == 2 ? defect_point2d<double>(a, a.phi, p)
                              : defect_point3d<double>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.acc, p, a.P, a.S);
    rho[p] = r;
    d[p] = 0.0;
    q[p] = 0.0;
    if (r32) r32[p] = (float)r;
    s = fma(r, r, s);
  }
  block_sum2(s, unused);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// partials of z . q and d . q (the previous direction)
template <int DIM, typename TZ>
__global__ void __launch_bounds__(kThreads) k_fcg_dots(Lvl<double> a, const TZ* __restrict__ z,
                                                      const double* __restrict__ d, const double* __restrict__ q,
                                                      double* parts) {
  pdl_enter();
  double zq = 0.0, dq = 0.0;
  JMG_FOR_GROUPS(a, kGroup<DIM>) {
    double zv[kGroup<DIM>], dv[kGroup<DIM>], qv[kGroup<DIM>];
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        zv[u] = (double)z[p];
        dv[u] = d[p];
        qv[u] = q[p];
      }
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        zq = fma(zv[u], qv[u], zq);
        dq = fma(dv[u], qv[u], dq);
      }
  }
  block_sum2(zq, dq);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = zq;
    parts[2 * blockIdx.x + 1] = dq;
  }
}

// beta from the dots; d <- z - beta d, q <- L z - beta q; partials of d . rho and d . q
template <int DIM, typename TZ>
__global__ void __launch_bounds__(kThreads) k_fcg_dir(Lvl<double> a, const TZ* z, double* d, double* q,
                                                     const double* rho, const double* parts_in, double* parts) {
  pdl_enter();
  double zq, dq;
  totals2(parts_in, &zq, &dq);
  const double beta = dq != 0.0 ? zq / dq : 0.0;
  double dr = 0.0, dqn = 0.0;
  JMG_FOR_POINTS(a, p) {
    const double dn = fma(-beta, d[p], (double)z[p]);
    const double qn = fma(-beta, q[p], apply_L<DIM, TZ>(a, z, p));
    d[p] = dn;
    q[p] = qn;
    dr = fma(dn, rho[p], dr);
    dqn = fma(dn, qn, dqn);
  }
  block_sum2(dr, dqn);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = dr;
    parts[2 * blockIdx.x + 1] = dqn;
  }
}

// alpha from the dots; x += alpha d, rho -= alpha q, r32 = float(rho); partials of rho . rho
template <int DIM>
__global__ void __launch_bounds__(kThreads) k_fcg_step(Lvl<double> a, const double* __restrict__ d,
                                                      const double* __restrict__ q, double* __restrict__ rho,
                                                      float* __restrict__ r32, const double* parts_in, double* parts) {
  pdl_enter();
  double dr, dq;
  totals2(parts_in, &dr, &dq);
  const double alpha = dq != 0.0 ? dr / dq : 0.0;
  double s = 0.0, unused = 0.0;
  double* __restrict__ x = a.phi;
  JMG_FOR_GROUPS(a, kGroup<DIM>) {
    double xv[kGroup<DIM>], dv[kGroup<DIM>], qv[kGroup<DIM>], rv[kGroup<DIM>];
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        xv[u] = x[p];
        dv[u] = d[p];
        qv[u] = q[p];
        rv[u] = rho[p];
      }
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        x[p] = fma(alpha, dv[u], xv[u]);
        const double r = fma(-alpha, qv[u], rv[u]);
        rho[p] = r;
        if (r32) r32[p] = (float)r;
        s = fma(r, r, s);
      }
  }
  block_sum2(s, unused);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// ---- mixed precision: FP32 directions, FP64 solution and true residual ----------------
// Inside FP64 refinement the search directions need only the preconditioner's accuracy:
// d and q = L d are kept in FP32 and built with the FP32 coefficient mirrors, the step
// x += alpha d is FP64, and the residual is recomputed exactly, rho = rhs - L x in FP64,
// every step (so the stopping test reads the true residual; no recurrence to drift).

// L z in FP32 with the FP32 coefficients (9-point terms when present)
template <int DIM>
__device__ __forceinline__ float apply_L32(const Lvl<float>& a, const float* z, long long p) {
  float t = a.acc[p] * z[p];
  t = fmaf(-a.wx[p - 1], z[p - 1], t);
  t = fmaf(-a.wx[p], z[p + 1], t);
  t = fmaf(-a.wy[p - a.P], z[p - a.P], t);
  t = fmaf(-a.wy[p], z[p + a.P], t);
  if (DIM == 3) {
    t = fmaf(-a.wz[p - a.S], z[p - a.S], t);
    t = fmaf(-a.wz[p], z[p + a.S], t);
  }
  if (DIM == 2 && a.xll) {
    const int P = a.P;
    float o = a.xll[p] * z[p - P - 1];
    o = fmaf(a.xrl[p], z[p - P + 1], o);
    o = fmaf(a.xlr[p], z[p + P - 1], o);
    o = fmaf(a.xrr[p], z[p + P + 1], o);
    t = t - o;
  }
  return -t;
}

// rho = rhs - L x (FP64), r32 = float(rho), d32 = q32 = 0; partials of rho . rho
template <int DIM>
__global__ void __launch_bounds__(kThreads) k_fcg32_init(Lvl<double> a, float* __restrict__ r32,
                                                        float* __restrict__ d, float* __restrict__ q,
                                                        double* parts) {
  pdl_enter();
  double s = 0.0, unused = 0.0;
  JMG_FOR_GROUPS(a, kGroupStencil<DIM>) {
    double r[kGroupStencil<DIM>];
#pragma unroll
    for (int u = 0; u < kGroupStencil<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        r[u] = DIM == 2 ? defect_point2d<double>(a, a.phi, p)
                        : defect_point3d<double>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.acc, p, a.P, a.S);
      }
#pragma unroll
    for (int u = 0; u < kGroupStencil<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        r32[p] = (float)r[u];
        if (d) {
          d[p] = 0.f;
          q[p] = 0.f;
        }
        s = fma(r[u], r[u], s);
      }
  }
  block_sum2(s, unused);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// partials of z . q and d . q (FP32 products, FP64 block sums)
template <int DIM>
__global__ void __launch_bounds__(kThreads, DIM == 3 ? 4 : 1) k_fcg32_dots(Lvl<double> a, const float* __restrict__ z,
                                                        const float* __restrict__ d, const float* __restrict__ q,
                                                        double* parts) {
  pdl_enter();
  float zq = 0.f, dq = 0.f;
  JMG_FOR_GROUPS(a, kGroup<DIM>) {
    float zv[kGroup<DIM>], dv[kGroup<DIM>], qv[kGroup<DIM>];
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        zv[u] = z[p];
        dv[u] = d[p];
        qv[u] = q[p];
      }
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        zq = fmaf(zv[u], qv[u], zq);
        dq = fmaf(dv[u], qv[u], dq);
      }
  }
  double a0 = zq, a1 = dq;
  block_sum2(a0, a1);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = a0;
    parts[2 * blockIdx.x + 1] = a1;
  }
}

// beta; d <- z - beta d, q <- L32 z - beta q (FP32); partials of d . r32 and d . q
template <int DIM>
__global__ void __launch_bounds__(kThreads) k_fcg32_dir(Lvl<double> a, Lvl<float> a32, const float* __restrict__ z,
                                                       float* __restrict__ d, float* __restrict__ q,
                                                       const float* __restrict__ r32, const double* parts_in,
                                                       double* parts) {
  pdl_enter();
  double zq, dq;
  totals2(parts_in, &zq, &dq);
  const float beta = dq != 0.0 ? (float)(zq / dq) : 0.f;
  float dr = 0.f, dqn = 0.f;
  JMG_FOR_GROUPS(a, kGroupStencil<DIM>) {
    float dn[kGroupStencil<DIM>], qn[kGroupStencil<DIM>], rv[kGroupStencil<DIM>];
#pragma unroll
    for (int u = 0; u < kGroupStencil<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        dn[u] = fmaf(-beta, d[p], z[p]);
        qn[u] = fmaf(-beta, q[p], apply_L32<DIM>(a32, z, p));
        rv[u] = r32[p];
      }
#pragma unroll
    for (int u = 0; u < kGroupStencil<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        d[p] = dn[u];
        q[p] = qn[u];
        dr = fmaf(dn[u], rv[u], dr);
        dqn = fmaf(dn[u], qn[u], dqn);
      }
  }
  double b0 = dr, b1 = dqn;
  block_sum2(b0, b1);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = b0;
    parts[2 * blockIdx.x + 1] = b1;
  }
}

// alpha; x += alpha d (FP64)
template <int DIM>
__global__ void __launch_bounds__(kThreads) k_fcg32_x(Lvl<double> a, const float* __restrict__ d,
                                                     const double* parts_in) {
  pdl_enter();
  double dr, dq;
  totals2(parts_in, &dr, &dq);
  const double alpha = dq != 0.0 ? dr / dq : 0.0;
  double* __restrict__ x = a.phi;
  JMG_FOR_GROUPS(a, kGroup<DIM>) {
    double xv[kGroup<DIM>];
    float dv[kGroup<DIM>];
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) {
        const long long p = base_[u] + i_;
        xv[u] = x[p];
        dv[u] = d[p];
      }
#pragma unroll
    for (int u = 0; u < kGroup<DIM>; ++u)
      if (u < n_) x[base_[u] + i_] = fma(alpha, (double)dv[u], xv[u]);
  }
}

}  // namespace

static int blocks_for(int dim, const Lvl<double>& a) {
  return fcg_blocks((a.my - 1) * (dim == 3 ? a.mz - 1 : 1));
}

int fcg_num_parts() { return kBlocks; }
int fcg_parts_used(int dim, const Lvl<double>& a) { return blocks_for(dim, a); }

void launch_fcg32_init(int dim, const Lvl<double>& a, float* r32, float* d, float* q, double* parts,
                       cudaStream_t s) {
  const int nb = blocks_for(dim, a);
  if (dim == 2) launch_k(k_fcg32_init<2>, dim3(nb), dim3(kThreads), 0, s, a, r32, d, q, parts);
  else launch_k(k_fcg32_init<3>, dim3(nb), dim3(kThreads), 0, s, a, r32, d, q, parts);
}

// one step after the cycle produced z (FP32): dots, directions, x update, true residual
void launch_fcg32_iter(int dim, const Lvl<double>& a, const Lvl<float>& a32, const float* z, float* d, float* q,
                       float* r32, double* parts_dots, double* parts_dir, double* parts_res, cudaStream_t s) {
  const int nb = blocks_for(dim, a);
  if (dim == 2) {
    launch_k(k_fcg32_dots<2>, dim3(nb), dim3(kThreads), 0, s, a, z, d, q, parts_dots);
    launch_k(k_fcg32_dir<2>, dim3(nb), dim3(kThreads), 0, s, a, a32, z, d, q, r32, parts_dots, parts_dir);
    launch_k(k_fcg32_x<2>, dim3(nb), dim3(kThreads), 0, s, a, d, parts_dir);
    launch_k(k_fcg32_init<2>, dim3(nb), dim3(kThreads), 0, s, a, r32, (float*)nullptr, (float*)nullptr,
             parts_res);
  } else {
    launch_k(k_fcg32_dots<3>, dim3(nb), dim3(kThreads), 0, s, a, z, d, q, parts_dots);
    launch_k(k_fcg32_dir<3>, dim3(nb), dim3(kThreads), 0, s, a, a32, z, d, q, r32, parts_dots, parts_dir);
    launch_k(k_fcg32_x<3>, dim3(nb), dim3(kThreads), 0, s, a, d, parts_dir);
    launch_k(k_fcg32_init<3>, dim3(nb), dim3(kThreads), 0, s, a, r32, (float*)nullptr, (float*)nullptr,
             parts_res);
  }
}

void launch_fcg_init(int dim, const Lvl<double>& a, double* rho, double* d, double* q, float* r32, double* parts,
                     cudaStream_t s) {
  const int nb = blocks_for(dim, a);
  if (dim == 2) launch_k(k_fcg_init<2>, dim3(nb), dim3(kThreads), 0, s, a, rho, d, q, r32, parts);
  else launch_k(k_fcg_init<3>, dim3(nb), dim3(kThreads), 0, s, a, rho, d, q, r32, parts);
}

template <typename TZ>
void launch_fcg_iter(int dim, const Lvl<double>& a, const TZ* z, double* d, double* q, double* rho, float* r32,
                     double* parts_dots, double* parts_dir, double* parts_res, cudaStream_t s) {
  const int nb = blocks_for(dim, a);
  if (dim == 2) {
    launch_k(k_fcg_dots<2, TZ>, dim3(nb), dim3(kThreads), 0, s, a, z, d, q, parts_dots);
    launch_k(k_fcg_dir<2, TZ>, dim3(nb), dim3(kThreads), 0, s, a, z, d, q, rho, parts_dots, parts_dir);
    launch_k(k_fcg_step<2>, dim3(nb), dim3(kThreads), 0, s, a, d, q, rho, r32, parts_dir, parts_res);
  } else {
    launch_k(k_fcg_dots<3, TZ>, dim3(nb), dim3(kThreads), 0, s, a, z, d, q, parts_dots);
    launch_k(k_fcg_dir<3, TZ>, dim3(nb), dim3(kThreads), 0, s, a, z, d, q, rho, parts_dots, parts_dir);
    launch_k(k_fcg_step<3>, dim3(nb), dim3(kThreads), 0, s, a, d, q, rho, r32, parts_dir, parts_res);
  }
}

template void launch_fcg_iter<float>(int, const Lvl<double>&, const float*, double*, double*, double*, float*,
                                     double*, double*, double*, cudaStream_t);
template void launch_fcg_iter<double>(int, const Lvl<double>&, const double*, double*, double*, double*, float*,
                                      double*, double*, double*, cudaStream_t);

}  // namespace jmg
