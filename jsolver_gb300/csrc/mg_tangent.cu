// mg_tangent.cu — forward mode of the fixed-mode 2D solve (Jacobian-vector product).
//
// The reference gets forward-mode derivatives from jax.jvp through its fixed loop
// (solver_2d.py:461-463). Here every quantity carries its tangent. The coefficient
// hierarchy (solver_2d.py:326-421) is linear in (lambda, D) except 1/A_cc, so the tangent
// hierarchy is the same hierarchy built from the tangent coefficients, with d(1/A_cc) =
// -(1/A_cc)^2 d(A_cc) replacing the reciprocal. The cycle is affine in (phi, rhs) for
// fixed coefficients; its tangent runs the same schedule with dual-number kernels:
//   sweep     phi' = (s - rhs) / A_cc,   s = sum of couplings x neighbours
//             dphi' = (ds - drhs) / A_cc + (s - rhs) d(1/A_cc),
//             ds = sum of (dcoupling x neighbour + coupling x dneighbour)
//   defect    d = A_cc phi - sum + rhs,  dd = dA_cc phi + A_cc dphi - dsum + drhs
//   restrict  linear in the defects (same weights for both)
//   prolong   linear (the grid-wide kernel applied to the tangent arrays)
// The tangent arrays live in a second workspace with the plan's own layout. Every level
// runs grid-wide kernels here (no single-block coarse kernel): the tangent is a test and
// analysis path, not the solver's hot loop.
#include <cuda_runtime.h>

#include "../../include/jmg.h"
#include "mg_kernels.h"
#include "mg_plan.h"

namespace jmg {

int set_error_message(int code, const char* msg);

namespace {

int fail(int code, const char* msg) { return set_error_message(code, msg); }

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// d(1/A_cc) = -(1/A_cc)^2 dA_cc over the whole level box (frames: 1/A_cc = 0 there)
__global__ void k_tan_invd(Lvl<double> a, Lvl<double> t) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I > a.mx + 2 || J > a.my + 2) return;
  const long long p = (long long)J * a.P + I;
  const double inv = a.invd[p];
  t.invd[p] = -(inv * inv) * t.acc[p];
}

// one colour of the dual sweep (solver_2d.py:670-692 with tangents)
__global__ void k_dual_sweep2d(Lvl<double> a, Lvl<double> t, int color) {
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 2;  // row
  if (i > a.my) return;
  const int j = 2 + ((i + color) & 1) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);  // column
  if (j > a.mx) return;
  const long long p = (long long)i * a.P + j;
  const int P = a.P;
  double s = a.wy[p] * a.phi[p + P];
  s = fma(a.wy[p - P], a.phi[p - P], s);
  s = fma(a.wx[p], a.phi[p + 1], s);
  s = fma(a.wx[p - 1], a.phi[p - 1], s);
  double ds = t.wy[p] * a.phi[p + P] + a.wy[p] * t.phi[p + P];
  ds += t.wy[p - P] * a.phi[p - P] + a.wy[p - P] * t.phi[p - P];
  ds += t.wx[p] * a.phi[p + 1] + a.wx[p] * t.phi[p + 1];
  ds += t.wx[p - 1] * a.phi[p - 1] + a.wx[p - 1] * t.phi[p - 1];
  const double r = s - a.rhs[p];
  a.phi[p] = r * a.invd[p];
  t.phi[p] = (ds - t.rhs[p]) * a.invd[p] + r * t.invd[p];
}

__device__ __forceinline__ void dual_defect(const Lvl<double>& a, const Lvl<double>& t, long long p, double* d,
                                            double* dd) {
  const int P = a.P;
  double v = a.acc[p] * a.phi[p];
  v = fma(-a.wx[p - 1], a.phi[p - 1], v);
  v = fma(-a.wx[p], a.phi[p + 1], v);
  v = fma(-a.wy[p - P], a.phi[p - P], v);
  v = fma(-a.wy[p], a.phi[p + P], v);
  *d = v + a.rhs[p];
  double w = t.acc[p] * a.phi[p] + a.acc[p] * t.phi[p];
  w -= t.wx[p - 1] * a.phi[p - 1] + a.wx[p - 1] * t.phi[p - 1];
  w -= t.wx[p] * a.phi[p + 1] + a.wx[p] * t.phi[p + 1];
  w -= t.wy[p - P] * a.phi[p - P] + a.wy[p - P] * t.phi[p - P];
  w -= t.wy[p] * a.phi[p + P] + a.wy[p] * t.phi[p + P];
  *dd = w + t.rhs[p];
}

// coarse rhs and its tangent from the red-point defects (solver_2d.py:616-647); coarse phi
// and its tangent set to zero, over the full padded coarse box
__global__ void k_dual_restrict2d(Lvl<double> af, Lvl<double> tf, Lvl<double> ac, Lvl<double> tc) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I > ac.mx + 2 || J > ac.my + 2) return;
  const long long q = (long long)J * ac.P + I;
  double v = 0.0, dv = 0.0;
  if (J >= 2 && J <= ac.my && I >= 2 && I <= ac.mx) {
    const int P = af.P;
    const long long c = (long long)(2 * J - 1) * P + (2 * I - 1);
    double dne, dnw, dse, dsw, dc, tne, tnw, tse, tsw, tc0;
    dual_defect(af, tf, c + P + 1, &dne, &tne);
    dual_defect(af, tf, c + P - 1, &dnw, &tnw);
    dual_defect(af, tf, c - P + 1, &dse, &tse);
    dual_defect(af, tf, c - P - 1, &dsw, &tsw);
    dual_defect(af, tf, c, &dc, &tc0);
    v = 0.0625 * (((dne + dnw) + dse) + dsw) + 0.25 * dc;
    dv = 0.0625 * (((tne + tnw) + tse) + tsw) + 0.25 * tc0;
  }
  ac.rhs[q] = v;
  ac.phi[q] = 0.0;
  tc.rhs[q] = dv;
  tc.phi[q] = 0.0;
}

void dual_sweep(const Lvl<double>& a, const Lvl<double>& t, cudaStream_t s) {
  dim3 b(64, 4), g(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4));
  for (int c = 0; c < 2; ++c) k_dual_sweep2d<<<g, b, 0, s>>>(a, t, c);
}

void dual_cycle(const JmgPlan* p, void* ws, void* tws, const CycleParams& cp, int lev, bool fcycle, bool skip_pre,
                cudaStream_t s) {
  const Lvl<double> a = lvl64(p, ws, lev), t = lvl64(p, tws, lev);
  if (lev == cp.last_level) {
    for (int k = 0; k < cp.nu1 + cp.nu2; ++k) dual_sweep(a, t, s);
    return;
  }
  if (!skip_pre)
    for (int k = 0; k < cp.nu1; ++k) dual_sweep(a, t, s);
  const Lvl<double> ac = lvl64(p, ws, lev + 1), tc = lvl64(p, tws, lev + 1);
  dim3 b(32, 8), g(cdiv(ac.mx + 3, 32), cdiv(ac.my + 3, 8));
  k_dual_restrict2d<<<g, b, 0, s>>>(a, t, ac, tc);
  if (fcycle)
    for (int k = 0; k < cp.gamma; ++k) dual_cycle(p, ws, tws, cp, lev + 1, true, false, s);
  for (int k = 0; k < cp.gamma; ++k) dual_cycle(p, ws, tws, cp, lev + 1, false, false, s);
  launch_prolong<double>(2, a, ac, cp.diag, s);
  launch_prolong<double>(2, t, tc, cp.diag, s);
  for (int k = 0; k < cp.nu2; ++k) dual_sweep(a, t, s);
}

}  // namespace
}  // namespace jmg

using namespace jmg;

extern "C" {

size_t jmg_tangent_workspace_bytes(const JmgPlan* p) { return p ? p->ws_bytes : 0; }

int jmg_solve_fixed_jvp(JmgPlan* p, const double* phi0, const double* rhs, const JmgCoeffs* c,
                        const double* phi0_dot, const double* rhs_dot, const JmgCoeffs* c_dot, double* phi_out,
                        double* phi_dot_out, void* ws, size_t ws_bytes, void* tws, size_t tws_bytes,
                        jmg_stream_t stream) {
  int rc = check_ws(p, ws, ws_bytes);
  if (rc) return rc;
  if ((rc = check_ws(p, tws, tws_bytes))) return rc;
  if (p->dim != 2) return fail(JMG_ERR_VALUE, "the tangent is implemented for 2D solves");
  if (!p->cfg.fixed) return fail(JMG_ERR_VALUE, "the tangent follows the fixed mode (fixed=True)");
  if (p->mixed || p->fcg || p->off_diag)
    return fail(JMG_ERR_VALUE, "the tangent differentiates the FP64 5-point iteration of the reference");
  if ((rc = check_coeffs(p, c))) return rc;
  if (!c_dot || !phi0 || !rhs || !phi0_dot || !rhs_dot || !phi_out || !phi_dot_out)
    return fail(JMG_ERR_VALUE, "NULL argument");
  for (int a = 0; a < 2; ++a)
    if ((c->D[a] == nullptr) != (c_dot->D[a] == nullptr))
      return fail(JMG_ERR_VALUE, "tangent D components must be arrays where D is, scalars where it is");
  if ((c->lam == nullptr) != (c_dot->lam == nullptr))
    return fail(JMG_ERR_VALUE, "the tangent of lambda must be an array where lambda is, a scalar where it is");
  cudaStream_t s = (cudaStream_t)stream;
  const Box b0 = p->lv[0].box;
  Lvl<double> a0 = lvl64(p, ws, 0), t0 = lvl64(p, tws, 0);
  // inputs; the frame of phi is zero at every cycle in fixed mode (solver_2d.py:462)
  launch_copy_in(b0, phi0, a0.phi, 1, s);
  launch_copy_in(b0, rhs, a0.rhs, 1, s);
  launch_copy_in(b0, phi0_dot, t0.phi, 1, s);
  launch_copy_in(b0, rhs_dot, t0.rhs, 1, s);
  // coefficients and their tangents (linear hierarchy; then d(1/A_cc))
  if ((rc = build_hierarchy(p, c, ws, s))) return rc;
  if ((rc = build_hierarchy(p, c_dot, tws, s))) return rc;
  for (int l = 0; l < p->used; ++l) {
    const Lvl<double> a = lvl64(p, ws, l), t = lvl64(p, tws, l);
    dim3 b(32, 8), g(cdiv(a.mx + 3, 32), cdiv(a.my + 3, 8));
    k_tan_invd<<<g, b, 0, s>>>(a, t);
  }
  const CycleParams cp = cycle_params(p, false);
  if (p->cfg.skip_pre)
    for (int k = 0; k < cp.nu1; ++k) dual_sweep(a0, t0, s);
  for (long long it = 0; it < p->cfg.max_iters_outer; ++it)
    dual_cycle(p, ws, tws, cp, 0, p->cfg.fcycle != 0, p->cfg.skip_pre != 0, s);
  launch_copy_out(b0, a0.phi, phi_out, s);
  launch_copy_out(b0, t0.phi, phi_dot_out, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(JMG_ERR_CUDA, cudaGetErrorString(e));
  return JMG_OK;
}

}  // extern "C"
