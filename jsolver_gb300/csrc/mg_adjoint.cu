// mg_adjoint.cu — hand-written reverse mode of the fixed-mode solve (vector-Jacobian
// product) in 2D (5- and 9-point stencils) and 3D, with per-cycle checkpointing and
// recomputation.
//
// The reference's fixed mode (solver_2d.py:461-463, solver_3d.py:468-470) is
// differentiated with jax.vjp, which tapes every cycle (memory grows with cycles x grid,
// performance.md:44-60). Here:
//   forward:  phi_0 (do_BCs) -> n cycles, keeping only phi at the start of every cycle;
//   backward: for k = n-1 .. 0: re-run cycle k from its checkpoint with per-operator
//             snapshots of phi, then apply the transposed operators in reverse order
//             (mg_adjoint_kernels.cu): colour updates reversed, restriction <-> prolongation
//             transposed; finally the backward of the coefficient hierarchy.
// Outputs: adjoints of phi0, rhs, lambda, the D components and D_xy (dense arrays, like
// the inputs). The
// frame of phi is reset by do_BCs at every sweep and cycle, so its adjoint there is zero.
// The checkpointed forward and the reverse sweep are captured once into a CUDA graph per
// (workspace, adjoint workspace) pair. Within a cycle, each run of operators on the small
// levels (at most 2048 points, below level 0) is one single-block launch forward (with its
// snapshots) and one in reverse (mg_adjoint_kernels.cu), instead of a few launches per
// operator.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/jmg.h"
#include "mg_adjoint_seg.h"
#include "mg_kernels.h"
#include "mg_plan.h"

namespace jmg {

void adj_sweep(int dim, const Lvl<double>& a, const AdjLvl& g, const double* before, const double* after,
               cudaStream_t s);
void adj_restrict(int dim, const Lvl<double>& a, const AdjLvl& g, const double* phi, const Lvl<double>& c,
                  const AdjLvl& gc, cudaStream_t s);
void adj_prolong(int dim, const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c, const AdjLvl& gc, int diag,
                 cudaStream_t s);
void adj_hierarchy2d(const Lvl<double>& a, const AdjLvl& g, int level, double sx, double sy, int nx0, double* dbx,
                     double* dby, double* dlam, cudaStream_t s);
void adj_hier_xy2d(const Lvl<double>& a, const AdjLvl& g, int level, double cxy, int nx0, double* dxy,
                   cudaStream_t s);
void adj_hierarchy3d(const Lvl<double>& a, const AdjLvl& g, int level, const double* sq, int nx0, int ny0,
                     const Lvl<double>* prev, double* const* gprev, const double* const* gcur, double* const* dbar,
                     double* dlam, cudaStream_t s);
int set_error_message(int code, const char* msg);

namespace {

enum { OP_SWEEP = kAdjOpSweep, OP_RESTRICT = kAdjOpRestrict, OP_PROLONG = kAdjOpProlong };
constexpr int kZeros = -1;  // phi of a coarse level right after the restriction zeroed it
constexpr int kInput = -2;  // phi of level 0 at the start of the cycle (the checkpoint)

struct TapeOp {
  int kind, lev, before, after;
};

struct Tape {
  std::vector<TapeOp> ops;
  std::vector<int> snap_lev;  // level of every snapshot
  // maximal runs [first, last] of operators on the small levels (at most 2048 padded
  // points, never level 0), each run by one block in one launch
  std::vector<std::pair<int, int>> segs;
};

// first level a single block takes: at most JMG_ADJ_BLOCK_POINTS padded points (2048 by
// default, the rule of the solve's coarse kernel), from level 1
int adj_block_start(const JmgPlan* p) {
  static const long long limit = [] {
    const char* e = getenv("JMG_ADJ_BLOCK_POINTS");
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? v : 2048LL;
  }();
  for (int l = 1; l < p->used; ++l) {
    const long long pts = (long long)p->lv[l].box.nx * p->lv[l].box.ny * p->lv[l].box.nz;
    if (pts <= limit) return l;
  }
  return p->used;  // none
}

void find_segments(const JmgPlan* p, Tape& t) {
  const int cs = adj_block_start(p);
  const int n = (int)t.ops.size();
  for (int k = 0; k < n;) {
    if (t.ops[k].lev < cs) {
      ++k;
      continue;
    }
    int e = k;
    while (e + 1 < n && t.ops[e + 1].lev >= cs) ++e;
    if (e - k + 1 <= kMaxSegOps) t.segs.push_back({k, e});  // longer runs stay grid-wide
    k = e + 1;
  }
}

// the forward schedule of one cycle (solver_2d.py:582-614), with the phi state each
// operator reads (before) and writes (after) as snapshot indices
void tape_cycle(const JmgPlan* p, Tape& t, std::vector<int>& cur, int lev, bool fcycle, bool skip_pre) {
  const CycleParams cp = cycle_params(p, p->off_diag);
  auto sweep = [&]() {
    const int after = (int)t.snap_lev.size();
    t.snap_lev.push_back(lev);
    t.ops.push_back({OP_SWEEP, lev, cur[lev], after});
    cur[lev] = after;
  };
  if (lev == cp.last_level) {
    for (int k = 0; k < cp.nu1 + cp.nu2; ++k) sweep();
    return;
  }
  if (!skip_pre)
    for (int k = 0; k < cp.nu1; ++k) sweep();
  t.ops.push_back({OP_RESTRICT, lev, cur[lev], -3});
  cur[lev + 1] = kZeros;
  if (fcycle)
    for (int g = 0; g < cp.gamma; ++g) tape_cycle(p, t, cur, lev + 1, true, false);
  for (int g = 0; g < cp.gamma; ++g) tape_cycle(p, t, cur, lev + 1, false, false);
  const int after = (int)t.snap_lev.size();
  t.snap_lev.push_back(lev);
  t.ops.push_back({OP_PROLONG, lev, cur[lev], after});
  cur[lev] = after;
  for (int k = 0; k < cp.nu2; ++k) sweep();
}

Tape make_tape(const JmgPlan* p) {
  Tape t;
  std::vector<int> cur(p->used, kZeros);
  cur[0] = kInput;
  tape_cycle(p, t, cur, 0, p->cfg.fcycle != 0, p->cfg.skip_pre != 0);
  find_segments(p, t);
  return t;
}

// adjoint arrays per level: pb, rb, T, gacc, the face gradients (2 or 3) and, with D_xy,
// the four diagonal-coupling gradients
int adj_arrays(const JmgPlan* p) { return 4 + p->dim + (p->off_diag ? 4 : 0); }

struct AdjLayout {
  size_t total = 0;
  std::vector<size_t> lvl;   // adj_arrays() arrays per level
  std::vector<size_t> snap;  // one level array per snapshot
  size_t ckpt = 0;           // (n + 1) level-0 arrays
  size_t zeros = 0;          // one level-0 array of zeros
  size_t pre = 0;            // skip_pre: phi after each initial sweep (nu1 level-0 arrays)
  size_t tabs = 0;           // AdjTables of the single-block segments
  size_t segs = 0;           // one AdjSeg per segment
  int ncyc = 0;
};

AdjLayout adj_layout(const JmgPlan* p, const Tape& t) {
  AdjLayout L;
  size_t off = 0;
  auto take = [&](size_t b) {
    const size_t o = off;
    off = align_up(off + b);
    return o;
  };
  for (int l = 0; l < p->used; ++l) L.lvl.push_back(take(adj_arrays(p) * p->lv[l].elems * 8));
  for (int lev : t.snap_lev) L.snap.push_back(take(p->lv[lev].elems * 8));
  L.ncyc = p->cfg.max_iters_outer > 0 ? (int)p->cfg.max_iters_outer : 0;
  L.ckpt = take((size_t)(L.ncyc + 1) * p->lv[0].elems * 8);
  L.zeros = take(p->lv[0].elems * 8);
  const int nu1 = p->cfg.nu1 > 0 ? p->cfg.nu1 : 0;
  L.pre = take((size_t)(p->cfg.skip_pre ? nu1 + 1 : 1) * p->lv[0].elems * 8);
  L.tabs = take(sizeof(AdjTables));
  L.segs = take(sizeof(AdjSeg) * (t.segs.empty() ? 1 : t.segs.size()));
  L.total = off;
  return L;
}

AdjLvl adj_lvl(const JmgPlan* p, void* aws, const AdjLayout& L, int l) {
  double* b = ptr<double>(aws, L.lvl[l]);
  const size_t n = p->lv[l].elems;
  AdjLvl g;
  memset(&g, 0, sizeof(g));
  g.pb = b;
  g.rb = b + n;
  g.T = b + 2 * n;
  g.gacc = b + 3 * n;
  g.gwx = b + 4 * n;
  g.gwy = b + 5 * n;
  double* q = b + 6 * n;
  if (p->dim == 3) {
    g.gwz = q;
    q += n;
  }
  if (p->off_diag) {
    g.gxll = q;
    g.gxrl = q + n;
    g.gxlr = q + 2 * n;
    g.gxrr = q + 3 * n;
  }
  return g;
}

int fail(int code, const char* m) { return set_error_message(code, m); }

#define JMG_ACUDA(call)                                                   \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) return fail(JMG_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// run the taped cycle forward on the workspace level arrays (phi_0 already loaded);
// with snapshots, copy phi of the level after every sweep / prolongation
void run_tape_forward(const JmgPlan* p, void* ws, void* aws, const AdjLayout& L, const Tape& t, bool snapshots,
                      cudaStream_t s) {
  const CycleParams cp = cycle_params(p, p->off_diag);
  // current buffer of every level (one-pass sweeps swap a level's two buffers)
  std::vector<Lvl<double>> cur(p->used);
  for (int l = 0; l < p->used; ++l) cur[l] = lvl64(p, ws, l);
  size_t next_seg = 0;
  for (int k = 0; k < (int)t.ops.size(); ++k) {
    if (next_seg < t.segs.size() && t.segs[next_seg].first == k) {  // a single-block run
      adj_seg_fwd(p->dim, ptr<AdjTables>(aws, L.tabs), ptr<AdjSeg>(aws, L.segs) + next_seg, snapshots, cp.diag, s);
      k = t.segs[next_seg].second;
      ++next_seg;
      continue;
    }
    const TapeOp& op = t.ops[k];
    Lvl<double>& a = cur[op.lev];
    if (op.kind == OP_SWEEP) launch_sweep<double>(p->dim, a, s);
    else if (op.kind == OP_RESTRICT) launch_restrict<double>(p->dim, a, cur[op.lev + 1], s);
    else launch_prolong<double>(p->dim, a, cur[op.lev + 1], cp.diag, s);
    if (snapshots && op.kind != OP_RESTRICT)
      cudaMemcpyAsync(ptr<double>(aws, L.snap[op.after]), a.phi, p->lv[op.lev].elems * 8, cudaMemcpyDeviceToDevice, s);
  }
  const Lvl<double> first = lvl64(p, ws, 0);
  if (cur[0].phi != first.phi)
    cudaMemcpyAsync(first.phi, cur[0].phi, p->lv[0].elems * 8, cudaMemcpyDeviceToDevice, s);
}

// the checkpointed forward (the one-off pre-smoothing, then n cycles keeping phi at the
// start of each) and the reverse sweep over the cycles, newest first. Reads and writes only
// the plan workspace ws and the adjoint workspace aws, so one capture serves every call
// with the same two addresses. phi_0, rhs and the hierarchy are in ws, the input adjoint in
// level 0's pb and every other adjoint array is zero when it starts.
void adj_core(const JmgPlan* p, void* ws, void* aws, const AdjLayout& L, const Tape& tape, cudaStream_t s) {
  const size_t e0 = p->lv[0].elems;
  Lvl<double> l0 = lvl64(p, ws, 0);
  const CycleParams cp = cycle_params(p, p->off_diag);
  const int nu1 = p->cfg.nu1 > 0 ? p->cfg.nu1 : 0;
  double* pre = ptr<double>(aws, L.pre);
  const double* zeros = ptr<double>(aws, L.zeros);
  // the single-block segments' tables and operators, their phi states resolved (segments
  // hold no level-0 operator, so no state depends on the cycle's checkpoint)
  if (!tape.segs.empty()) {
    AdjTables tabs;
    memset(&tabs, 0, sizeof(tabs));
    for (int l = 0; l < p->used; ++l) {
      tabs.lv.l[l] = lvl64(p, ws, l);
      tabs.g[l] = adj_lvl(p, aws, L, l);
    }
    adj_store_tables(tabs, ptr<AdjTables>(aws, L.tabs), s);
    for (size_t q = 0; q < tape.segs.size(); ++q) {
      AdjSeg sg;
      memset(&sg, 0, sizeof(sg));
      sg.n = tape.segs[q].second - tape.segs[q].first + 1;
      for (int k = 0; k < sg.n; ++k) {
        const TapeOp& op = tape.ops[tape.segs[q].first + k];
        AdjSegOp& o = sg.op[k];
        o.kind = op.kind;
        o.lev = op.lev;
        o.before = op.before == kZeros ? zeros : op.before >= 0 ? ptr<double>(aws, L.snap[op.before]) : nullptr;
        o.after = op.kind != OP_RESTRICT ? ptr<double>(aws, L.snap[op.after]) : nullptr;
      }
      adj_store_seg(sg, ptr<AdjSeg>(aws, L.segs) + q, s);
    }
  }
  if (p->cfg.skip_pre) {  // the one-off pre-smoothing (solver_2d.py:457-459)
    cudaMemcpyAsync(pre, l0.phi, e0 * 8, cudaMemcpyDeviceToDevice, s);
    Lvl<double> cur = l0;
    for (int k = 0; k < nu1; ++k) {
      launch_sweep<double>(p->dim, cur, s);
      cudaMemcpyAsync(pre + (size_t)(k + 1) * e0, cur.phi, e0 * 8, cudaMemcpyDeviceToDevice, s);
    }
    if (cur.phi != l0.phi) cudaMemcpyAsync(l0.phi, cur.phi, e0 * 8, cudaMemcpyDeviceToDevice, s);
  }
  double* ck = ptr<double>(aws, L.ckpt);
  for (int k = 0; k < L.ncyc; ++k) {
    // the loop body starts with do_BCs (solver_2d.py:462); the level-0 frame is already zero
    cudaMemcpyAsync(ck + (size_t)k * e0, l0.phi, e0 * 8, cudaMemcpyDeviceToDevice, s);
    run_tape_forward(p, ws, aws, L, tape, false, s);
  }
  std::vector<AdjLvl> g(p->used);
  for (int l = 0; l < p->used; ++l) g[l] = adj_lvl(p, aws, L, l);
  for (int k = L.ncyc - 1; k >= 0; --k) {
    cudaMemcpyAsync(l0.phi, ck + (size_t)k * e0, e0 * 8, cudaMemcpyDeviceToDevice, s);
    run_tape_forward(p, ws, aws, L, tape, true, s);
    auto state = [&](int idx) -> const double* {
      if (idx == kZeros) return zeros;
      if (idx == kInput) return ck + (size_t)k * e0;
      return ptr<double>(aws, L.snap[idx]);
    };
    int seg = (int)tape.segs.size() - 1;
    for (int t = (int)tape.ops.size() - 1; t >= 0; --t) {
      if (seg >= 0 && tape.segs[seg].second == t) {  // a single-block run, in reverse
        adj_seg_rev(p->dim, ptr<AdjTables>(aws, L.tabs), ptr<AdjSeg>(aws, L.segs) + seg, cp.diag, s);
        t = tape.segs[seg].first;
        --seg;
        continue;
      }
      const TapeOp& op = tape.ops[t];
      Lvl<double> a = lvl64(p, ws, op.lev);
      if (op.kind == OP_SWEEP) {
        adj_sweep(p->dim, a, g[op.lev], state(op.before), state(op.after), s);
      } else if (op.kind == OP_PROLONG) {
        adj_prolong(p->dim, a, g[op.lev], lvl64(p, ws, op.lev + 1), g[op.lev + 1], cp.diag, s);
      } else {
        adj_restrict(p->dim, a, g[op.lev], state(op.before), lvl64(p, ws, op.lev + 1), g[op.lev + 1], s);
      }
    }
  }
  if (p->cfg.skip_pre)
    for (int k = nu1 - 1; k >= 0; --k)
      adj_sweep(p->dim, l0, g[0], pre + (size_t)k * e0, pre + (size_t)(k + 1) * e0, s);
}

}  // namespace
}  // namespace jmg

using namespace jmg;

extern "C" {

size_t jmg_adjoint_workspace_bytes(const JmgPlan* p) {
  if (!p) return 0;
  return adj_layout(p, make_tape(p)).total;
}

int jmg_solve_fixed_vjp_nd(JmgPlan* p, const double* phi0, const double* rhs, const JmgCoeffs* c,
                           const double* phi_bar, double* phi0_bar, double* rhs_bar, double* lam_bar,
                           double* const* D_bar, double* Dxy_bar, void* ws, size_t ws_bytes, void* aws,
                           size_t aws_bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, ws_bytes);
  if (rc) return rc;
  if (!p->cfg.fixed) return fail(JMG_ERR_VALUE, "reverse mode needs fixed mode (as in the reference)");
  if (p->mixed) return fail(JMG_ERR_VALUE, "the adjoint differentiates the FP64 method (precision fp64)");
  if (p->fcg) return fail(JMG_ERR_VALUE, "the adjoint differentiates the reference's iteration (outer richardson)");
  if ((rc = check_coeffs(p, c))) return rc;
  const int dim = p->dim;
  if (!c->lam || !D_bar) return fail(JMG_ERR_VALUE, "the adjoint needs lambda and D as arrays (broadcast scalars first)");
  for (int a = 0; a < dim; ++a)
    if (!c->D[a] || !D_bar[a])
      return fail(JMG_ERR_VALUE, "the adjoint needs lambda and D as arrays (broadcast scalars first)");
  if (p->off_diag && !Dxy_bar) return fail(JMG_ERR_VALUE, "a plan with D_xy needs the D_xy adjoint output");
  if (!phi0 || !rhs || !phi_bar || !phi0_bar || !rhs_bar || !lam_bar) return fail(JMG_ERR_VALUE, "NULL array argument");
  const Tape tape = make_tape(p);
  const AdjLayout L = adj_layout(p, tape);
  if (!aws || aws_bytes < L.total || reinterpret_cast<uintptr_t>(aws) % kAlign)
    return fail(JMG_ERR_WORKSPACE, "adjoint workspace missing, too small or misaligned");
  cudaStream_t s = (cudaStream_t)stream;
  const Box b0 = p->lv[0].box;
  const size_t dense = (size_t)b0.nx * b0.ny * b0.nz;
  Lvl<double> l0 = lvl64(p, ws, 0);

  // the input adjoint and the zeroed adjoint state, then the checkpointed forward and the
  // reverse sweep (one graph launch, or the same operations from the host)
  launch_copy_in(b0, phi0, l0.phi, 1, s);
  launch_copy_in(b0, rhs, l0.rhs, 1, s);
  if ((rc = build_hierarchy(p, c, ws, s))) return rc;
  JMG_ACUDA(cudaMemsetAsync(aws, 0, L.total, s));
  launch_copy_in(b0, phi_bar, adj_lvl(p, aws, L, 0).pb, 1, s);  // the output's frame is a constant (do_BCs)
  if (p->host_loop) {
    adj_core(p, ws, aws, L, tape, s);
  } else {
    if (!p->vjp_exec || p->vjp_ws != ws || p->vjp_aws != aws) {
      if (p->vjp_exec) {
        cudaGraphExecDestroy(p->vjp_exec);
        p->vjp_exec = nullptr;
      }
      if (!p->cap) JMG_ACUDA(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
      JMG_ACUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
      adj_core(p, ws, aws, L, tape, p->cap);
      cudaGraph_t graph = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(p->cap, &graph);
      JMG_ACUDA(ec);
      cudaGraphExec_t exec = nullptr;
      const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      JMG_ACUDA(ei);
      p->vjp_exec = exec;
      p->vjp_ws = ws;
      p->vjp_aws = aws;
    }
    JMG_ACUDA(cudaGraphLaunch(p->vjp_exec, s));
  }
  const AdjLvl g0 = adj_lvl(p, aws, L, 0);

  // adjoints of the inputs: phi0, rhs (level 0), then the coefficient hierarchy
  launch_copy_out(b0, g0.pb, phi0_bar, s);
  launch_copy_out(b0, g0.rb, rhs_bar, s);
  JMG_ACUDA(cudaMemsetAsync(lam_bar, 0, dense * 8, s));
  for (int a = 0; a < dim; ++a) JMG_ACUDA(cudaMemsetAsync(D_bar[a], 0, dense * 8, s));
  if (p->off_diag) JMG_ACUDA(cudaMemsetAsync(Dxy_bar, 0, dense * 8, s));
  if (dim == 2) {
    for (int l = 0; l < p->used; ++l) {
      const double ix = p->grid.idel[0] * std::pow(0.5, l), iy = p->grid.idel[1] * std::pow(0.5, l);
      const Lvl<double> a = lvl64(p, ws, l);
      const AdjLvl g = adj_lvl(p, aws, L, l);
      adj_hierarchy2d(a, g, l, ix * ix, iy * iy, b0.nx, D_bar[0], D_bar[1], lam_bar, s);
      if (p->off_diag) adj_hier_xy2d(a, g, l, (ix * iy) * 0.25, b0.nx, Dxy_bar, s);
    }
  } else {
    // the chained 3D hierarchy, coarsest level first. pb, rb and T of the levels >= 1 are
    // free after the reverse sweep and hold the adjoints of their averaged D (zeroed here).
    for (int l = 1; l < p->used; ++l) JMG_ACUDA(cudaMemsetAsync(adj_lvl(p, aws, L, l).pb, 0, 3 * p->lv[l].elems * 8, s));
    for (int l = p->used - 1; l >= 0; --l) {
      double sq[3];
      for (int a = 0; a < 3; ++a) {
        const double id = p->grid.idel[a] * std::pow(0.5, l);
        sq[a] = id * id;
      }
      const AdjLvl g = adj_lvl(p, aws, L, l);
      const double* gcur[3] = {g.T, g.pb, g.rb};
      double* gprev[3] = {nullptr, nullptr, nullptr};
      Lvl<double> prev;
      if (l >= 2) {
        const AdjLvl gp = adj_lvl(p, aws, L, l - 1);
        gprev[0] = gp.T;
        gprev[1] = gp.pb;
        gprev[2] = gp.rb;
        prev = lvl64(p, ws, l - 1);
      }
      adj_hierarchy3d(lvl64(p, ws, l), g, l, sq, b0.nx, b0.ny, l >= 2 ? &prev : nullptr, l >= 2 ? gprev : nullptr,
                      l >= 1 ? gcur : nullptr, D_bar, lam_bar, s);
    }
  }
  JMG_ACUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_solve_fixed_vjp(JmgPlan* p, const double* phi0, const double* rhs, const JmgCoeffs* c, const double* phi_bar,
                        double* phi0_bar, double* rhs_bar, double* lam_bar, double* Dxx_bar, double* Dyy_bar,
                        void* ws, size_t ws_bytes, void* aws, size_t aws_bytes, jmg_stream_t stream) {
  if (p && p->dim != 2) return fail(JMG_ERR_VALUE, "jmg_solve_fixed_vjp is the 2D form (jmg_solve_fixed_vjp_nd: 3D)");
  if (p && p->off_diag) return fail(JMG_ERR_VALUE, "jmg_solve_fixed_vjp has no D_xy output (jmg_solve_fixed_vjp_nd)");
  double* D_bar[3] = {Dxx_bar, Dyy_bar, nullptr};
  return jmg_solve_fixed_vjp_nd(p, phi0, rhs, c, phi_bar, phi0_bar, rhs_bar, lam_bar, D_bar, nullptr, ws, ws_bytes,
                                aws, aws_bytes, stream);
}

}  // extern "C"
