// mg_tile2d.cu — shared-memory tiled 2D kernels that compute every fine value once:
// the defect + restriction onto the next level and the FP64 residual of a refinement step.
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_dual.cuh"

namespace jmg {

// ---------------------------------------------------------------------------------------
// FP64 side of a refinement step (mixed precision): r = rhs - L_h phi in FP64, stored as
// FP32 for the next FP32 cycle, and per-block partial sums of r^2 (fixed tile-to-block
// map and fixed in-block order, so the norm is reproducible). The correction itself is
// added to phi by the last FP32 sweep (acc64 above).
// ---------------------------------------------------------------------------------------

constexpr int kRX = 64, kRY = 16;

int residual_f32_parts2d(int mx, int my) { return ((mx - 1 + kRX - 1) / kRX) * ((my - 1 + kRY - 1) / kRY); }

__global__ void __launch_bounds__(256) k_residual_f32_2d(Lvl<double> a, float* __restrict__ r32,
                                                         double* __restrict__ parts) {
  pdl_enter();
  __shared__ double Phi[kRY + 2][kRX + 2];  // rows i0-1 .. i0+RY, columns j0-1 .. j0+RX
  __shared__ double red[8];
  const int i0 = 2 + blockIdx.y * kRY, j0 = 2 + blockIdx.x * kRX;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const long long P = a.P;
  for (int t = tid; t < (kRY + 2) * (kRX + 2); t += 256) {
    const int r = t / (kRX + 2), q = t % (kRX + 2);
    const int i = i0 - 1 + r, j = j0 - 1 + q;
    double v = 0.0;
    if (i <= a.my + 2 && j <= a.mx + 2) v = a.phi[i * P + j];
    Phi[r][q] = v;
  }
  __syncthreads();
  double sum = 0.0;
  for (int rr = 0; rr < kRY / 8; ++rr) {
    for (int cc = 0; cc < kRX / 32; ++cc) {
      const int i = i0 + threadIdx.y + 8 * rr, j = j0 + threadIdx.x + 32 * cc;
      if (i > a.my || j > a.mx) continue;
      const int r = i - i0 + 1, q = j - j0 + 1;
      const long long p = i * P + j;
      // same operation order as defect_point2d
      double d = a.acc[p] * Phi[r][q];
      d = fma(-a.wx[p - 1], Phi[r][q - 1], d);
      d = fma(-a.wx[p], Phi[r][q + 1], d);
      d = fma(-a.wy[p - P], Phi[r - 1][q], d);
      d = fma(-a.wy[p], Phi[r + 1][q], d);
      d = d + a.rhs[p];
      r32[p] = (float)d;
      sum = fma(d, d, sum);
    }
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (threadIdx.x == 0) red[threadIdx.y] = sum;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w];
    parts[blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

void launch_residual_f32_2d(const Lvl<double>& a, float* r32, double* parts, cudaStream_t s) {
  dim3 b(32, 8), g((unsigned)((a.mx - 1 + kRX - 1) / kRX), (unsigned)((a.my - 1 + kRY - 1) / kRY));
  launch_k(k_residual_f32_2d, g, b, 0, s, a, r32, parts);
}


// ---------------------------------------------------------------------------------------
// Defect + restriction onto level+1 (solver_2d.py:616-647), each fine defect computed once.
// A block owns a TJ x TI tile of coarse indices (frame included: frame values are 0). The
// coarse point (J, I) reads the defects at its centre (2J-1, 2I-1) and at the four
// diagonal neighbours (2J-1 +- 1, 2I-1 +- 1), all red points; neighbouring coarse points
// share the diagonal ones. The block stages phi on the fine footprint plus a one-point
// halo, computes the defects of the footprint's red points once into shared memory, then
// forms 1/16 (ne + nw + se + sw) + 1/4 centre in the reference's order. Also phi_c = 0.
// ---------------------------------------------------------------------------------------

constexpr int kCJ = 8, kCI = 32;                            // coarse points per block
constexpr int kDR = 2 * kCJ + 1, kDC = 2 * kCI + 1;         // fine defect footprint
constexpr int kFR = kDR + 2, kFC = kDC + 2;                  // with the one-point halo

template <typename T>
__global__ void __launch_bounds__(256) k_restrict_tile2d(Lvl<T> f, Lvl<T> c) {
  pdl_enter();
  constexpr int NT = 256;
  __shared__ T Phi[kFR][kFC];
  __shared__ T Def[kDR][kDC];
  const int J0 = blockIdx.y * kCJ, I0 = blockIdx.x * kCI;
  const int fr0 = 2 * J0 - 2, fc0 = 2 * I0 - 2;  // fine index of Def[0][0]
  const int tid = threadIdx.x;
  const long long P = f.P;
  // Every thread issues all its loads of a phase before using them: on the small levels
  // these kernels are latency-bound, and one load per loop iteration made each phase
  // wait once per iteration.
  constexpr int U1 = (kFR * kFC + NT - 1) / NT;
  {
    T v[U1];
#pragma unroll
    for (int u = 0; u < U1; ++u) {
      const int t = tid + u * NT;
      v[u] = T(0);
      if (t < kFR * kFC) {
        const int r = t / kFC, q = t - r * kFC;
        const int i = fr0 - 1 + r, j = fc0 - 1 + q;
        if (i >= 0 && j >= 0 && i <= f.my + 2 && j <= f.mx + 2) v[u] = f.phi[i * P + j];
      }
    }
#pragma unroll
    for (int u = 0; u < U1; ++u) {
      const int t = tid + u * NT;
      if (t < kFR * kFC) (&Phi[0][0])[t] = v[u];
    }
  }
  __syncthreads();
  constexpr int XR = (kDC + 1) / 2;  // red candidates per footprint row
  constexpr int NRED = kDR * XR;
  constexpr int U2 = (NRED + NT - 1) / NT;
  {
    T ac[U2], wxm[U2], wxp[U2], wym[U2], wyp[U2], rh[U2];
    int pos[U2];
#pragma unroll
    for (int u = 0; u < U2; ++u) {
      const int t = tid + u * NT;
      pos[u] = -1;
      if (t < NRED) {
        const int r = t / XR, xp = t - r * XR;
        const int i = fr0 + r;
        const int q = 2 * xp + ((i + fc0) & 1);  // j = fc0 + q has i + j even (red)
        const int j = fc0 + q;
        if (q < kDC && i >= 2 && i <= f.my && j >= 2 && j <= f.mx) {
          const long long p = i * P + j;
          pos[u] = r * kDC + q;
          ac[u] = f.acc[p];
          wxm[u] = f.wx[p - 1];
          wxp[u] = f.wx[p];
          wym[u] = f.wy[p - P];
          wyp[u] = f.wy[p];
          rh[u] = f.rhs[p];
        }
      }
    }
    // the non-red entries of Def are never read; the red ones outside the interior are 0
#pragma unroll
    for (int u = 0; u < U2; ++u) {
      const int t = tid + u * NT;
      if (t >= NRED) continue;
      const int r = t / XR, xp = t - r * XR;
      const int i = fr0 + r;
      const int q = 2 * xp + ((i + fc0) & 1);
      if (q >= kDC) continue;
      T d = T(0);
      if (pos[u] >= 0) {
        const int rr = r + 1, qq = q + 1;  // position in Phi
        // same operation order as defect_point2d
        d = ac[u] * Phi[rr][qq];
        d = fma(-wxm[u], Phi[rr][qq - 1], d);
        d = fma(-wxp[u], Phi[rr][qq + 1], d);
        d = fma(-wym[u], Phi[rr - 1][qq], d);
        d = fma(-wyp[u], Phi[rr + 1][qq], d);
        d = d + rh[u];
      }
      Def[r][q] = d;
    }
  }
  __syncthreads();
  const long long Pc = c.P;
  for (int t = tid; t < kCJ * kCI; t += NT) {
    const int J = J0 + t / kCI, I = I0 + t % kCI;
    if (J > c.my + 2 || I > c.mx + 2) continue;
    T v = T(0);
    if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) {
      const int r = 2 * J - 1 - fr0, q = 2 * I - 1 - fc0;
      const T s = ((Def[r + 1][q + 1] + Def[r + 1][q - 1]) + Def[r - 1][q + 1]) + Def[r - 1][q - 1];
      v = T(0.0625) * s + T(0.25) * Def[r][q];
    }
    c.rhs[J * Pc + I] = v;
    c.phi[J * Pc + I] = T(0);
  }
}

template <typename T>
void launch_restrict_tile2d(const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  dim3 g((unsigned)((c.mx + 3 + kCI - 1) / kCI), (unsigned)((c.my + 3 + kCJ - 1) / kCJ));
  launch_k(k_restrict_tile2d<T>, g, dim3(256), 0, s, f, c);
}

// phi_f += P phi_c (solver_2d.py:649-668) by coarse cells: a thread takes the fine rows
// 2J-1 .. 2J and columns 2I-1 .. 2I, which interpolate from the four coarse corners
// (J .. J+1, I .. I+1); it loads those once and forms each fine value with
// prolong_point2d's formula for its class, in the same order (bit-identical to
// k_prolong2d); the (even, even) points only with diag (nu2 <= 0 or D_xy).
template <typename T>
__global__ void __launch_bounds__(256) k_prolong2d_cells(Lvl<T> f, Lvl<T> c, int diag) {
  pdl_enter();
  const int I = 1 + blockIdx.x * blockDim.x + threadIdx.x;  // coarse column, 1 .. m_c
  const int J = 1 + blockIdx.y * blockDim.y + threadIdx.y;  // coarse row
  if (I > c.mx || J > c.my) return;
  prolong_cell2d<T>(f, c, J, I, diag != 0);
}

template <typename T>
void launch_prolong_cells2d(const Lvl<T>& f, const Lvl<T>& c, int diag, cudaStream_t s) {
  dim3 b(32, 8), g((unsigned)((c.mx + 31) / 32), (unsigned)((c.my + 7) / 8));
  launch_k(k_prolong2d_cells<T>, g, b, 0, s, f, c, diag);
}

template void launch_prolong_cells2d<double>(const Lvl<double>&, const Lvl<double>&, int, cudaStream_t);
template void launch_prolong_cells2d<float>(const Lvl<float>&, const Lvl<float>&, int, cudaStream_t);
// the forward-mode solve (mg_tangent.cu)
template void launch_prolong_cells2d<Dual>(const Lvl<Dual>&, const Lvl<Dual>&, int, cudaStream_t);

template void launch_restrict_tile2d<double>(const Lvl<double>&, const Lvl<double>&, cudaStream_t);
template void launch_restrict_tile2d<float>(const Lvl<float>&, const Lvl<float>&, cudaStream_t);

}  // namespace jmg
