// mg_tangent.cu — forward mode of the solve (Jacobian-vector product), 2D and 3D, fixed
// and dynamic, 5-, 7- and 9-point stencils.
//
// The reference gets forward-mode derivatives from jax.jvp through its solve: through the
// fixed fori_loop (solver_2d.py:461-463) and through the dynamic while_loop (465-477),
// whose cycle count is not differentiated: the loop runs as many cycles as the primal's
// distance test asks for and the tangent rides along (tests/test_solver_2d.py:173-176,
// tests/test_solver_3d.py:208-211 check it on every problem). Here every quantity is a
// dual number (mg_dual.cuh) and the cycle runs the solver's own kernels over Duals:
//   coefficients  the hierarchy (solver_2d.py:326-421, solver_3d.py:338-429) is linear in
//                 (lambda, D, D_xy) except 1/A_cc, so the tangent hierarchy is the plan's
//                 hierarchy built from the tangent coefficients, with
//                 (1/A_cc)' = -(1/A_cc)^2 A_cc'; value and tangent arrays are packed into
//                 Dual arrays per level;
//   cycle         colour sweeps (sub-lattice passes with D_xy), the one-thread-per-coarse-
//                 point restriction, the prolongation by coarse cells and the single-block
//                 coarse cycle, all instantiated for Dual;
//   loop          fixed: max_iters_outer cycles; dynamic: the reference's distance test on
//                 the value part (max |phi_old - phi| over the padded box, NaN ends it),
//                 decided on the device by the solver's loop kernel and read back by the
//                 host after every cycle.
// The value part is the plain FP64 solver's arithmetic, so phi and the cycle count are
// jmg_solve's bit for bit. The tangent workspace holds the tangent hierarchy in the plan's
// layout, then the Dual level arrays, the distance snapshot and the loop state.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/jmg.h"
#include "mg_dual.cuh"
#include "mg_kernels.h"
#include "mg_plan.h"

namespace jmg {

namespace {

int fail(int code, const char* msg) { return set_error_message(code, msg); }

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Dual arrays of a level: phi, rhs, wx, wy, [wz], invd, acc, [A_ll, A_rl, A_lr, A_rr]
int dual_arrays(const JmgPlan* p) { return (p->dim == 3 ? 7 : 6) + (p->off_diag ? 4 : 0); }

struct TanLayout {
  std::vector<size_t> lvl;  // first Dual array of every level
  size_t phi_old = 0;       // FP64 level-0 snapshot of the distance test
  size_t state = 0;         // LoopState
  size_t tab = 0;           // LvlTable<Dual> of the coarse kernel
  size_t total = 0;
};

TanLayout tan_layout(const JmgPlan* p) {
  TanLayout L;
  size_t off = align_up(p->ws_bytes);  // the tangent hierarchy, in the plan's layout
  auto take = [&](size_t b) {
    const size_t o = off;
    off = align_up(off + b);
    return o;
  };
  for (int l = 0; l < p->used; ++l) L.lvl.push_back(take((size_t)dual_arrays(p) * p->lv[l].elems * sizeof(Dual)));
  L.phi_old = take(p->lv[0].elems * 8);
  L.state = take(sizeof(LoopState));
  L.tab = take(sizeof(LvlTable<Dual>));
  L.total = off;
  return L;
}

Lvl<Dual> dual_lvl(const JmgPlan* p, void* tws, const TanLayout& L, int l) {
  const LevelInfo& li = p->lv[l];
  const size_t n = li.elems;
  Dual* b = ptr<Dual>(tws, L.lvl[l]);
  Lvl<Dual> a{};
  int k = 0;
  a.phi = b + n * k++;
  a.rhs = b + n * k++;
  a.wx = b + n * k++;
  a.wy = b + n * k++;
  a.wz = p->dim == 3 ? b + n * k++ : nullptr;
  a.invd = b + n * k++;
  a.acc = b + n * k++;
  if (p->off_diag) {
    a.xll = b + n * k++;
    a.xrl = b + n * k++;
    a.xlr = b + n * k++;
    a.xrr = b + n * k++;
  }
  a.mx = li.m[0];
  a.my = li.m[1];
  a.mz = li.m[2];
  a.P = li.box.P;
  a.S = li.box.S;
  a.phi2 = nullptr;
  return a;
}

// out = (v, t) over the pitched box; with invd, out = (v, -v^2 t): t is A_cc' and v 1/A_cc
__global__ void k_pack_dual(Box b, const double* __restrict__ v, const double* __restrict__ t, Dual* __restrict__ out,
                            int invd) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  const long long p = (long long)K * b.S + (long long)J * b.P + I;
  const double x = v[p], y = t[p];
  out[p] = invd ? Dual(x, -(x * x) * y) : Dual(x, y);
}

// dense (value, tangent) -> pitched Duals; the frame is zeroed (do_BCs) with zero_frame
__global__ void k_dual_copy_in(Box b, const double* __restrict__ v, const double* __restrict__ t,
                               Dual* __restrict__ out, int zero_frame) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  const long long q = ((long long)K * b.ny + J) * b.nx + I;
  Dual x(v[q], t[q]);
  if (zero_frame) {
    const bool fr = I < 2 || I >= b.nx - 2 || J < 2 || J >= b.ny - 2 || (b.nz > 1 && (K < 2 || K >= b.nz - 2));
    if (fr) x = Dual(0.0, 0.0);
  }
  out[(long long)K * b.S + (long long)J * b.P + I] = x;
}

__global__ void k_dual_copy_out(Box b, const Dual* __restrict__ in, double* __restrict__ v, double* __restrict__ t) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= b.nx || J >= b.ny) return;
  const Dual x = in[(long long)K * b.S + (long long)J * b.P + I];
  const long long q = ((long long)K * b.ny + J) * b.nx + I;
  v[q] = x.v;
  t[q] = x.d;
}

// distance of the value part (solver_2d.py:481-494: max |phi_old - phi| over the padded
// box, as ordered bits so that NaN propagates), then phi_old <- phi
__global__ void k_dual_distance(Box b, double* __restrict__ old_phi, const Dual* __restrict__ phi, LoopState* st) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  unsigned long long m = 0;
  if (I < b.nx && J < b.ny) {
    const long long p = (long long)K * b.S + (long long)J * b.P + I;
    const double n = phi[p].v;
    m = abs_bits(old_phi[p] - n);
    old_phi[p] = n;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
    m = w > m ? w : m;
  }
  if ((threadIdx.x & 31) == 0 && m) atomicMax(&st->dist_bits, m);
}

dim3 box_grid(const Box& b) { return dim3(cdiv(b.nx, 32), cdiv(b.ny, 8), b.nz); }

// multigrid_cycle (solver_2d.py:582-614, solver_3d.py:588-620) over Duals: grid-wide
// operators above the first coarse level, one single-block launch from there down
void dual_cycle(const JmgPlan* p, const LvlTable<Dual>& t, const LvlTable<Dual>* dt, const CycleParams& cp, int cs,
                int lev, bool fcycle, bool skip_pre, cudaStream_t s) {
  if (lev >= cs) {
    launch_coarse_cycle<Dual>(p->dim, dt, cp, lev, fcycle ? 1 : 0, skip_pre ? 1 : 0, s);
    return;
  }
  Lvl<Dual> a = t.l[lev];
  if (lev == cp.last_level) {
    for (int k = 0; k < cp.nu1 + cp.nu2; ++k) launch_sweep<Dual>(p->dim, a, s);
    return;
  }
  if (!skip_pre)
    for (int k = 0; k < cp.nu1; ++k) launch_sweep<Dual>(p->dim, a, s);
  launch_restrict_grid<Dual>(p->dim, a, t.l[lev + 1], s);
  if (fcycle)
    for (int g = 0; g < cp.gamma; ++g) dual_cycle(p, t, dt, cp, cs, lev + 1, true, false, s);
  for (int g = 0; g < cp.gamma; ++g) dual_cycle(p, t, dt, cp, cs, lev + 1, false, false, s);
  if (p->dim == 2) launch_prolong_cells2d<Dual>(a, t.l[lev + 1], cp.diag, s);
  else launch_prolong_cells3d<Dual>(a, t.l[lev + 1], cp.diag, s);
  for (int k = 0; k < cp.nu2; ++k) launch_sweep<Dual>(p->dim, a, s);
}

bool same_forms(const JmgPlan* p, const JmgCoeffs* c, const JmgCoeffs* d) {
  if ((c->lam == nullptr) != (d->lam == nullptr)) return false;
  for (int a = 0; a < p->dim; ++a)
    if ((c->D[a] == nullptr) != (d->D[a] == nullptr)) return false;
  return true;
}

}  // namespace
}  // namespace jmg

using namespace jmg;

extern "C" {

size_t jmg_tangent_workspace_bytes(const JmgPlan* p) { return p ? tan_layout(p).total : 0; }

int jmg_solve_jvp(JmgPlan* p, const double* phi0, const double* rhs, const JmgCoeffs* c, const double* phi0_dot,
                  const double* rhs_dot, const JmgCoeffs* c_dot, double* phi_out, double* phi_dot_out,
                  int64_t* count_out, void* ws, size_t ws_bytes, void* tws, size_t tws_bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, ws_bytes);
  if (rc) return rc;
  const TanLayout L = tan_layout(p);
  if (!tws || tws_bytes < L.total || reinterpret_cast<uintptr_t>(tws) % kAlign != 0)
    return fail(JMG_ERR_WORKSPACE, "tangent workspace missing, unaligned or smaller than jmg_tangent_workspace_bytes");
  if (p->mixed || p->fcg)
    return fail(JMG_ERR_VALUE, "the tangent differentiates the reference's FP64 iteration (precision fp64, outer "
                               "richardson)");
  if (!p->cfg.fixed && p->cfg.stop != JMG_STOP_DISTANCE)
    return fail(JMG_ERR_VALUE, "the tangent follows the reference's loops: fixed=True or the distance stop");
  if ((rc = check_coeffs(p, c))) return rc;
  if (!c_dot) return fail(JMG_ERR_VALUE, "coeffs_dot must not be NULL");
  if ((rc = check_coeffs(p, c_dot))) return rc;
  if (!same_forms(p, c, c_dot))
    return fail(JMG_ERR_VALUE, "tangents of lambda and D must be arrays where lambda and D are arrays, scalars "
                               "where they are scalars");
  if (!phi0 || !rhs || !phi0_dot || !rhs_dot || !phi_out || !phi_dot_out) return fail(JMG_ERR_VALUE, "NULL argument");
  if ((rc = coarse_setup(p))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const Box b0 = p->lv[0].box;
  // coefficients and their tangents: the plan's hierarchy of c in ws and of c_dot in tws,
  // packed into Duals ((1/A_cc)' = -(1/A_cc)^2 A_cc')
  if ((rc = build_hierarchy(p, c, ws, s))) return rc;
  if ((rc = build_hierarchy(p, c_dot, tws, s))) return rc;
  LvlTable<Dual> tab;
  memset(&tab, 0, sizeof(tab));
  for (int l = 0; l < p->used; ++l) {
    const Lvl<double> a = lvl64(p, ws, l), t = lvl64(p, tws, l);
    const Lvl<Dual> d = dual_lvl(p, tws, L, l);
    const Box& b = p->lv[l].box;
    const dim3 g = box_grid(b), blk(32, 8, 1);
    k_pack_dual<<<g, blk, 0, s>>>(b, a.wx, t.wx, d.wx, 0);
    k_pack_dual<<<g, blk, 0, s>>>(b, a.wy, t.wy, d.wy, 0);
    if (p->dim == 3) k_pack_dual<<<g, blk, 0, s>>>(b, a.wz, t.wz, d.wz, 0);
    k_pack_dual<<<g, blk, 0, s>>>(b, a.acc, t.acc, d.acc, 0);
    k_pack_dual<<<g, blk, 0, s>>>(b, a.invd, t.acc, d.invd, 1);
    if (p->off_diag) {
      k_pack_dual<<<g, blk, 0, s>>>(b, a.xll, t.xll, d.xll, 0);
      k_pack_dual<<<g, blk, 0, s>>>(b, a.xrl, t.xrl, d.xrl, 0);
      k_pack_dual<<<g, blk, 0, s>>>(b, a.xlr, t.xlr, d.xlr, 0);
      k_pack_dual<<<g, blk, 0, s>>>(b, a.xrr, t.xrr, d.xrr, 0);
    }
    tab.l[l] = d;
  }
  LvlTable<Dual>* dtab = ptr<LvlTable<Dual>>(tws, L.tab);
  launch_store_table<Dual>(tab, dtab, s);
  // inputs; phi_old keeps phi0 with its frame (the first distance sees it, solver_2d.py:471)
  Lvl<Dual> d0 = tab.l[0];
  double* phi_old = ptr<double>(tws, L.phi_old);
  LoopState* st = ptr<LoopState>(tws, L.state);
  k_dual_copy_in<<<box_grid(b0), dim3(32, 8, 1), 0, s>>>(b0, phi0, phi0_dot, d0.phi, 1);
  k_dual_copy_in<<<box_grid(b0), dim3(32, 8, 1), 0, s>>>(b0, rhs, rhs_dot, d0.rhs, 1);
  launch_copy_in(b0, phi0, phi_old, 0, s);
  const CycleParams cp = cycle_params(p, p->off_diag);
  // the coarse kernel of the solve: the single block from the same level as jmg_solve's
  const int cs = p->cluster_ranks ? block_coarse_level(p) : p->coarse_start;
  const int mode = p->cfg.fixed ? 2 : 0;
  // skip_pre: pre-smoothing once, before the loop (solver_2d.py:457-459)
  const bool presmoothed = p->cfg.skip_pre && cp.nu1 > 0;
  if (presmoothed) {
    for (int k = 0; k < cp.nu1; ++k) launch_sweep<Dual>(p->dim, d0, s);
    k_dual_distance<<<box_grid(b0), dim3(32, 8, 1), 0, s>>>(b0, phi_old, d0.phi, st);  // phi_old <- smoothed phi
  }
  const bool runs = p->cfg.max_iters_outer > 0;
  if (runs) {
    launch_loop_init(st, nullptr, 0, mode, p->cfg.rtol, p->cfg.max_iters_outer, 0, s);
    if (mode == 2) {
      for (long long it = 0; it < p->cfg.max_iters_outer; ++it)
        dual_cycle(p, tab, dtab, cp, cs, 0, p->cfg.fcycle != 0, p->cfg.skip_pre != 0, s);
    } else {
      for (;;) {
        int go = 0;
        cudaError_t e = cudaMemcpyAsync(&go, &st->go, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(JMG_ERR_CUDA, cudaGetErrorString(e));
        if (!go) break;
        dual_cycle(p, tab, dtab, cp, cs, 0, p->cfg.fcycle != 0, p->cfg.skip_pre != 0, s);
        k_dual_distance<<<box_grid(b0), dim3(32, 8, 1), 0, s>>>(b0, phi_old, d0.phi, st);
        launch_loop_step(st, nullptr, 0, mode, p->cfg.epsilon, p->cfg.rtol, p->cfg.max_iters_outer, 0, s);
      }
    }
  }
  // outputs; with no cycle and no smoothing phi0 and its tangent come back untouched
  const size_t dense = (size_t)b0.nx * b0.ny * b0.nz * 8;
  if (runs || presmoothed) {
    k_dual_copy_out<<<box_grid(b0), dim3(32, 8, 1), 0, s>>>(b0, d0.phi, phi_out, phi_dot_out);
  } else {
    if (phi_out != phi0) cudaMemcpyAsync(phi_out, phi0, dense, cudaMemcpyDeviceToDevice, s);
    if (phi_dot_out != phi0_dot) cudaMemcpyAsync(phi_dot_out, phi0_dot, dense, cudaMemcpyDeviceToDevice, s);
  }
  if (count_out) {
    if (mode == 2 || !runs) {
      const long long n = runs ? p->cfg.max_iters_outer : 0;
      cudaMemcpyAsync(count_out, &n, sizeof(n), cudaMemcpyHostToDevice, s);
      cudaStreamSynchronize(s);  // n lives on this stack frame
    } else {
      launch_count_out(st, (long long*)count_out, s);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(JMG_ERR_CUDA, cudaGetErrorString(e));
  return JMG_OK;
}

int jmg_solve_fixed_jvp(JmgPlan* p, const double* phi0, const double* rhs, const JmgCoeffs* c,
                        const double* phi0_dot, const double* rhs_dot, const JmgCoeffs* c_dot, double* phi_out,
                        double* phi_dot_out, void* ws, size_t ws_bytes, void* tws, size_t tws_bytes,
                        jmg_stream_t stream) {
  if (p && !p->cfg.fixed) return fail(JMG_ERR_VALUE, "jmg_solve_fixed_jvp needs a plan with fixed = 1");
  return jmg_solve_jvp(p, phi0, rhs, c, phi0_dot, rhs_dot, c_dot, phi_out, phi_dot_out, nullptr, ws, ws_bytes, tws,
                       tws_bytes, stream);
}

}  // extern "C"
