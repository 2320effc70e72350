// mg_driver.cu — plan, workspace layout, cycle schedule, CUDA graph and the C ABI.
//
// A solve (Solver_2D.solve, solver_2d.py:423-479; Solver_3D.solve, solver_3d.py:431-486)
// runs as:
//   1. copy phi0 / rhs from the caller's dense arrays into the pitched level-0 arrays
//   2. coefficient hierarchy (mg_hierarchy.cu), one pass pair per level
//   3. optional pre-smoothing (skip_pre, solver_2d.py:457-459)
//   4. one launch of a CUDA graph: [loop init] -> WHILE(cond) { cycle; distance or
//      residual; loop step }. The cycle is the reference's recursion (solver_2d.py:582-614)
//      unrolled on the host into grid-wide kernel launches for the fine levels and one
//      single-block kernel for every visit of the first coarse level, exactly as the JIT
//      trace of the reference unrolls it into XLA ops.
//   5. copy phi back to the caller's dense array; the cycle count goes to a device int64.
// The graph is captured once per (plan, workspace address) and cached in the plan.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/jmg.h"
#include "mg_kernels.h"
#include "mg_plan.h"

using namespace jmg;

namespace {

thread_local std::string g_last_error;

int set_err(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define JMG_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return set_err(JMG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// First level run by the single-block global-memory coarse kernel: at most 2048 padded
// points (2D 32^2, 3D 8^3 interiors), and never below the last visited level. Thresholds
// of 256 to 8192 points measured on GB300: 2048 is fastest for the 2D and 3D solves in
// FP64 and in mixed precision; at 8192 the block spends longer on the 64^2 / 16^3 level
// than one grid-wide launch per operator takes.
long long coarse_block_points() {
  static const long long limit = [] {
    const char* e = getenv("JMG_COARSE_POINTS");  // tuning knob; 2048 by default
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? v : 2048LL;
  }();
  return limit;
}

int block_coarse_start(const JmgPlan* p) {
  const long long limit = coarse_block_points();
  for (int l = 0; l < p->used; ++l) {
    const long long pts = (long long)p->lv[l].box.nx * p->lv[l].box.ny * p->lv[l].box.nz;
    if (pts <= limit) return l;
  }
  return p->used - 1;
}

int validate_and_layout(JmgPlan* p) {
  const JmgGrid& g = p->grid;
  if (p->cfg.outer != JMG_OUTER_RICHARDSON && p->cfg.outer != JMG_OUTER_FCG)
    return set_err(JMG_ERR_VALUE, "outer must be JMG_OUTER_RICHARDSON or JMG_OUTER_FCG, got %d", p->cfg.outer);
  if (p->cfg.outer == JMG_OUTER_FCG && !p->cfg.fixed && p->cfg.stop != JMG_STOP_RESIDUAL)
    return set_err(JMG_ERR_VALUE, "outer='fcg' needs stop='residual' or fixed=True (the distance test "
                                  "measures a stationary iteration)");
  if (g.ndim != 2 && g.ndim != 3) return set_err(JMG_ERR_VALUE, "ndim must be 2 or 3, got %d", g.ndim);
  const char* names[3] = {"x", "y", "z"};
  const int d = g.ndim;
  // power-of-two checks in x, y, z order (solver_2d.py:292-295; solver_3d.py:295-300)
  for (int a = 0; a < d; ++a) {
    const long long m = g.m[a];
    if (m <= 0 || (m & (m - 1)) != 0)
      return set_err(JMG_ERR_VALUE, "Resolution of %s-grid is not a power of 2. Value: %lld", names[a], m);
  }
  int lv[3];
  int L = 1 << 30;
  for (int a = 0; a < d; ++a) {
    lv[a] = (int)std::ceil(std::log2((double)g.m[a])) + 1;
    L = lv[a] < L ? lv[a] : L;
  }
  // efficiency checks (solver_2d.py:304-307; solver_3d.py:312-317)
  for (int a = 0; a < d; ++a) {
    const long long coarsest = 1LL << (lv[a] - L);
    if (coarsest > 5)
      return set_err(JMG_ERR_VALUE,
                     "Resolution of %s-grid not efficient for multigrid configuration. Resolution of coarsest level: %lld",
                     names[a], coarsest);
  }
  // linear grids only (solver_2d.py:320-321; solver_3d.py:331-332)
  for (int a = 0; a < d; ++a)
    if (!g.is_linear[a]) return set_err(JMG_ERR_VALUE, "Only linear grids are supported!");
  if (L < 2)
    return set_err(JMG_ERR_VALUE,
                   "Resolution too small for multigrid: the smallest axis needs at least 2 cells (got levels=%d)", L);
  if (L > kMaxLevels + 1) return set_err(JMG_ERR_VALUE, "too many levels (%d)", L);
  p->dim = d;
  p->levels = L;
  p->used = L - 1;
  p->mixed = p->cfg.precision == JMG_PREC_MIXED;
  if (p->cfg.off_diag && d != 2) return set_err(JMG_ERR_VALUE, "off_diag (D_xy) is a 2D option");
  p->off_diag = d == 2 && p->cfg.off_diag;
  p->lv.resize(p->used);
  // one-pass sweeps (mg_fused.cu, mg_sweep_tma3d.cu), 5- and 7-point stencils: the 3D
  // levels whose one-pass grid fills at least half a wave of the GPU (256^3 levels and
  // finer) and the 2D grid-wide levels (more points than the coarse block takes; they
  // run the sweeps beyond the fused pairs' two, e.g. the four extra post-sweeps of a
  // V(1,5) cycle: 2D 1024^2 mixed + FCG 5.65 against 5.79 ms; JMG_FUSED2D=0 turns the 2D
  // ones off); with JMG_FUSED_POINTS set, every level of at least that many padded points.
  // These levels get a second phi buffer. FP32 levels by default, FP64 levels too with
  // JMG_FUSED64=1; JMG_FUSED=0 turns them off.
  const long long fused_min = [] {
    const char* e = getenv("JMG_FUSED_POINTS");
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? v : 0LL;
  }();
  const char* fe = getenv("JMG_FUSED");
  const char* fe64 = getenv("JMG_FUSED64");
  const bool fused_on = !p->off_diag && !(fe && fe[0] == '0');
  const bool fused64 = fused_on && fe64 && fe64[0] == '1';
  const char* fe2 = getenv("JMG_FUSED2D");
  const bool fused2d = !(fe2 && fe2[0] == '0');
  // fused operator pairs on the levels the grid-wide kernels run (more points than the
  // single-block coarse kernel takes): 2D (mg_fusedops2d.cu, 5-point stencil) by default,
  // JMG_FUSEDOPS=0 turns them off; 3D (mg_fusedops3d.cu) only with JMG_FUSEDOPS3D=1, since
  // they measured no faster there (3D 256^3 mixed + FCG 95.2 against 94.8 ms, plain FP64
  // 1316 against 1280 ms: within a graph the small levels' launches already overlap, and
  // the halos add FP64 work)
  const char* fo = getenv("JMG_FUSEDOPS");
  const char* fo3 = getenv("JMG_FUSEDOPS3D");
  const bool fuseops_on =
      !p->off_diag && !(fo && fo[0] == '0') && (d == 2 || (fo3 && fo3[0] == '1'));
  const long long block_limit = coarse_block_points();
  // Largest fused level (padded points): every FP32 level, FP64 levels up to 2^19 points.
  // On larger FP64 levels the halos' extra FP64 work outweighs the saved launches (2D
  // 1024^2 plain FP64, measured: 40.7 ms with the 512^2 level and below fused, 43.5 ms
  // with level 0 too, 42.0 ms unfused; mixed + FCG 6.97 ms all fused, 7.73 ms unfused).
  // JMG_FUSEDOPS_MAX overrides it.
  // 3D: levels up to 2^19 padded points (64^3 and smaller), where launches are bound by
  // latency; on larger ones the halos' recomputation (about 3.5 sweeps' work per owned
  // point) outweighs the saved launches. JMG_FUSEDOPS_MAX overrides both.
  const long long fuse_max = [&] {
    const char* e = getenv("JMG_FUSEDOPS_MAX");
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? v : ((p->mixed && d == 2) ? (1LL << 62) : (1LL << 19));
  }();
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  for (int l = 0; l < p->used; ++l) {
    LevelInfo& li = p->lv[l];
    for (int a = 0; a < 3; ++a) li.m[a] = a < d ? (int)(g.m[a] >> l) : 0;
    li.box.nx = li.m[0] + 3;
    li.box.ny = li.m[1] + 3;
    li.box.nz = d == 3 ? li.m[2] + 3 : 1;
    li.box.P = (li.box.nx + 15) / 16 * 16;
    li.box.S = (long long)li.box.P * li.box.ny;
    li.elems = (size_t)li.box.S * li.box.nz;
    const size_t b8 = li.elems * 8, b4 = li.elems * 4;
    li.phi = take(b8);
    li.rhs = take(b8);
    li.wx = take(b8);
    li.wy = take(b8);
    li.wz = d == 3 ? take(b8) : 0;
    li.invd = take(b8);
    li.acc = take(b8);
    for (int c = 0; c < 4; ++c) li.xd[c] = li.xd32[c] = 0;
    if (p->off_diag)
      for (int c = 0; c < 4; ++c) li.xd[c] = take(b8);
    for (int c = 0; c < 3; ++c) li.d[c] = (d == 3 && l >= 1) ? take(b8) : 0;
    const bool fused_level =
        fused_on && li.elems < (1ULL << 31) &&  // the one-pass kernels index with 32 bits
        (fused_min > 0 ? (long long)li.elems >= fused_min
                       : d == 3 ? fused_wave_permille(li.m[0], li.m[1], li.m[2]) >= 500
                                : fused2d && (long long)li.box.nx * li.box.ny > block_limit);
    li.onepass64 = fused_level && fused64;
    li.onepass32 = fused_level && p->mixed;
    const long long pts = (long long)li.box.nx * li.box.ny * li.box.nz;
    li.fuse_ops = fuseops_on && l + 1 < p->used && pts > block_limit && pts <= fuse_max;
    li.phi2 = li.onepass64 || (li.fuse_ops && !p->mixed) ? take(b8) : 0;
    li.phi2_32 = 0;
    if (p->mixed) {
      if (li.onepass32 || li.fuse_ops) li.phi2_32 = take(b4);
      li.phi32 = take(b4);
      li.rhs32 = take(b4);
      li.wx32 = take(b4);
      li.wy32 = take(b4);
      li.wz32 = d == 3 ? take(b4) : 0;
      li.invd32 = take(b4);
      li.acc32 = take(b4);
      if (p->off_diag)
        for (int c = 0; c < 4; ++c) li.xd32[c] = take(b4);
    }
  }
  p->off_phi_old = take(p->lv[0].elems * 8);
  p->off_state = take(sizeof(LoopState));
  p->nparts = residual_num_parts(d, p->lv[0].box);
  {
    const int fused_parts = d == 2 ? residual_f32_parts2d(p->lv[0].m[0], p->lv[0].m[1]) : 0;
    const int maxparts = p->nparts > fused_parts ? p->nparts : fused_parts;
    p->off_parts = take((size_t)maxparts * 8 + 64);
  }
  p->off_tab64 = take(sizeof(LvlTable<double>));
  p->off_tab32 = take(sizeof(LvlTable<float>));
  p->fcg = p->cfg.outer == JMG_OUTER_FCG;
  if (p->fcg) {
    // FP64 cycles: FP64 rho, d, q, z; mixed: FP32 d, q (x and the true residual are FP64)
    const size_t b8 = p->lv[0].elems * 8, bv = p->lv[0].elems * (p->mixed ? 4 : 8);
    p->off_rho = p->mixed ? 0 : take(b8);
    p->off_d = take(bv);
    p->off_q = take(bv);
    p->off_z64 = p->mixed ? 0 : take(b8);
    p->off_fcg_parts = take((size_t)fcg_num_parts() * 5 * 8);
    p->off_tab64z = take(sizeof(LvlTable<double>));
  }
  p->ws_bytes = off;
  // the coarse levels are chosen at the first solve (coarse_setup), when the GPU's
  // cluster support is known; until then the single-block rule holds
  p->coarse_start = block_coarse_start(p);
  {
    // JMG_COARSE=cluster selects the thread-block-cluster coarse kernel; the default is
    // the single-block kernel, measured as fast or faster at every size on GB300
    const char* cm = getenv("JMG_COARSE");
    p->force_block = !(cm && std::strcmp(cm, "cluster") == 0);
  }
  const char* hl = getenv("JMG_HOST_LOOP");
  p->host_loop = hl && hl[0] == '1';
  return JMG_OK;
}


}  // namespace
// The persistent middle-level kernel (mg_mid2d.cu), opt-in with JMG_MID=1, for 2D 5-point
// plans with nu1, nu2 >= 1 whose coarse sub-cycle runs on the staged single block: it
// takes over from the first level below level 0 with at most JMG_MID_POINTS padded points
// (2^19 by default: 512^2 and smaller), provided every level from there to the coarse
// block runs the fused operator pairs in the precision of the cycles (FP32 with mixed
// precision, else FP64). JMG_MID_STALL=1 is the test mode whose first grid barrier never
// completes. The operation list of the longest cycle form must fit kMaxMidOps, or the
// kernel starts one level lower. Measured on GB300 it is slower than the separate
// launches it replaces (2D 1024^2 mixed + FCG 9.6 against 6.3 ms; one launch 107 us
// against about 49 us of launches per cycle): a grid-wide barrier costs more than a
// kernel boundary with programmatic dependent launch, so it is not the default.
static void mid_setup(JmgPlan* p) {
  p->mid_start = -1;
  p->mid_smem64 = p->mid_smem32 = 0;
  p->mid_blocks = 0;
  const char* me = getenv("JMG_MID");
  const char* mp = getenv("JMG_MID_POINTS");
  const char* ms = getenv("JMG_MID_STALL");
  p->mid_stall = ms && ms[0] == '1';
  const long long mid_max = (mp && atoll(mp) > 0) ? atoll(mp) : (1LL << 19);
  const size_t staged = p->mixed ? p->coarse_staged32 : p->coarse_staged64;
  if (!(me && me[0] == '1') || p->dim != 2 || p->off_diag || p->cluster_ranks || p->coarse_smem32 || !staged ||
      p->cfg.nu1 < 1 || p->cfg.nu2 < 1 || p->coarse_start < 2)
    return;
  const CycleParams cp = cycle_params(p, false);
  for (int l = 1; l < p->coarse_start; ++l) {
    const LevelInfo& li = p->lv[l];
    const long long pts = (long long)li.box.nx * li.box.ny;
    if (pts > mid_max) continue;
    bool fused = true;
    for (int k = l; k < p->coarse_start; ++k) {
      const LevelInfo& lk = p->lv[k];
      // (the kernel runs a level's sweeps beyond the fused pairs as its own colour passes,
      // whatever the level's one-pass flag: the same bits)
      fused = fused && lk.fuse_ops && (p->mixed ? lk.phi2_32 != 0 : lk.phi2 != 0);
    }
    if (!fused) continue;
    MidOps ops;
    if (!mid_ops(cp, p->coarse_start, l, p->cfg.fcycle != 0, true, &ops)) continue;
    int blocks = 0;
    const size_t smem = p->mixed ? prepare_mid2d<float>(staged, &blocks) : prepare_mid2d<double>(staged, &blocks);
    if (!smem) return;
    (p->mixed ? p->mid_smem32 : p->mid_smem64) = smem;
    p->mid_blocks = blocks;
    p->mid_start = l;
    return;
  }
}

// How the coarse levels of a cycle run. By default one block runs the levels of at most
// 2048 points from global memory. With JMG_COARSE=cluster (and cluster support) a
// thread-block cluster of 16 CTAs (8 where 16 is not allowed) takes every level from
// the first one of at most 20 000 padded points whose rows, with the levels below, fit
// in 200 KB of shared memory per CTA. On GB300 the coarse levels are bound by the
// latency of short FP64 dependency chains, not by one SM's FP64 rate, so the cluster
// gains nothing (measured per cycle: 2D 1024^2 180 us cluster vs 176 us block).
int jmg::coarse_setup(JmgPlan* p) {
  if (p->coarse_ready) return JMG_OK;
  const int last = p->used - 1;
  const int dim = p->dim;
  int m[kMaxLevels][3];
  for (int l = 0; l < p->used && l < kMaxLevels; ++l)
    for (int a = 0; a < 3; ++a) m[l][a] = p->lv[l].m[a];
  const size_t limit = 200 * 1024;
  p->cluster_ranks = 0;
  p->coarse_start = block_coarse_start(p);
  if (!p->force_block && !p->off_diag && p->used <= kMaxLevels) {
    for (int ranks : {16, 8}) {
      int lev0 = -1;
      ClusterLayout lay;
      for (int l = 0; l <= last; ++l) {
        const long long pts = (long long)p->lv[l].box.nx * p->lv[l].box.ny * p->lv[l].box.nz;
        if (pts > 20000) continue;
        if (cluster_layout(dim, m, l, last, ranks, &lay)) continue;
        if ((size_t)lay.elems * 8 > limit) continue;
        lev0 = l;
        break;
      }
      if (lev0 < 0) continue;
      const size_t b64 = (size_t)lay.elems * 8, b32 = (size_t)lay.elems * 4;
      if (prepare_coarse_cluster<double>(dim, b64, ranks)) continue;
      if (p->mixed && prepare_coarse_cluster<float>(dim, b32, ranks)) continue;
      p->cluster = lay;
      p->cluster_ranks = ranks;
      p->cluster_smem64 = b64;
      p->cluster_smem32 = b32;
      p->coarse_start = lev0;
      break;
    }
  }
  // The single block stages its levels in shared memory unless JMG_COARSE=global asks for
  // the global-memory kernel; JMG_COARSE_THREADS sets its block size (512 by default).
  p->coarse_staged64 = p->coarse_staged32 = 0;
  {
    const char* cg = getenv("JMG_COARSE");
    const char* ct = getenv("JMG_COARSE_THREADS");
    const int nt = ct ? atoi(ct) : 0;
    p->coarse_threads = (nt >= 64 && nt <= 512 && nt % 32 == 0) ? nt : 512;
    if (!p->cluster_ranks && !(cg && std::strcmp(cg, "global") == 0) && p->used <= kMaxLevels) {
      size_t elems[kMaxLevels];
      for (int l = 0; l < p->used; ++l) elems[l] = p->lv[l].elems;
      const size_t b64 = coarse_staged_bytes(dim, elems, p->coarse_start, last, 8, p->off_diag);
      if (b64 && prepare_coarse_staged<double>(dim, b64) == 0) p->coarse_staged64 = b64;
      const size_t b32 = coarse_staged_bytes(dim, elems, p->coarse_start, last, 4, p->off_diag);
      if (p->mixed && b32 && prepare_coarse_staged<float>(dim, b32) == 0) p->coarse_staged32 = b32;
    }
  }
  p->coarse_smem32 = 0;
  const char* c32 = getenv("JMG_COARSE32");
  // opt-in (JMG_COARSE32=smem): staging ~150 KB per launch costs more than the L2 round
  // trips it saves (2D 1024^2 mixed + FCG: 10.87 ms with it, 10.32 ms without)
  if (p->mixed && dim == 2 && !p->off_diag && !p->cluster_ranks && c32 && std::strcmp(c32, "smem") == 0) {
    int mx[kMaxLevels], my[kMaxLevels];
    for (int l = 0; l < p->used && l < kMaxLevels; ++l) {
      mx[l] = p->lv[l].m[0];
      my[l] = p->lv[l].m[1];
    }
    const size_t b = coarse_smem32_bytes(mx, my, p->coarse_start, last);
    if (b <= 200 * 1024 && prepare_coarse_smem32(b) == 0) p->coarse_smem32 = b;
  }
  prepare_fused_ops2d();  // kernel attributes, set outside any stream capture
  prepare_fused_ops3d();
  if (p->dim == 3 && p->mixed) sweep_tma3d_ready();
  mid_setup(p);
  cudaGetLastError();  // a refused attribute or occupancy query leaves no sticky error
  p->coarse_ready = true;
  return JMG_OK;
}

Lvl<double> jmg::lvl64(const JmgPlan* p, void* ws, int l) {
  const LevelInfo& li = p->lv[l];
  Lvl<double> a{};
  a.phi = ptr<double>(ws, li.phi);
  if (p->off_diag) {
    a.xll = ptr<double>(ws, li.xd[0]);
    a.xrl = ptr<double>(ws, li.xd[1]);
    a.xlr = ptr<double>(ws, li.xd[2]);
    a.xrr = ptr<double>(ws, li.xd[3]);
  }
  a.rhs = ptr<double>(ws, li.rhs);
  a.wx = ptr<double>(ws, li.wx);
  a.wy = ptr<double>(ws, li.wy);
  a.wz = p->dim == 3 ? ptr<double>(ws, li.wz) : nullptr;
  a.invd = ptr<double>(ws, li.invd);
  a.acc = ptr<double>(ws, li.acc);
  a.phi2 = li.phi2 ? ptr<double>(ws, li.phi2) : nullptr;
  a.onepass = li.onepass64 ? 1 : 0;
  a.fuseops = li.fuse_ops && li.phi2 ? 1 : 0;
  a.mx = li.m[0];
  a.my = li.m[1];
  a.mz = li.m[2];
  a.P = li.box.P;
  a.S = li.box.S;
  return a;
}
namespace {

}  // namespace
Lvl<float> jmg::lvl32(const JmgPlan* p, void* ws, int l) {
  const LevelInfo& li = p->lv[l];
  Lvl<float> a{};
  a.phi = ptr<float>(ws, li.phi32);
  if (p->off_diag) {
    a.xll = ptr<float>(ws, li.xd32[0]);
    a.xrl = ptr<float>(ws, li.xd32[1]);
    a.xlr = ptr<float>(ws, li.xd32[2]);
    a.xrr = ptr<float>(ws, li.xd32[3]);
  }
  a.rhs = ptr<float>(ws, li.rhs32);
  a.wx = ptr<float>(ws, li.wx32);
  a.wy = ptr<float>(ws, li.wy32);
  a.wz = p->dim == 3 ? ptr<float>(ws, li.wz32) : nullptr;
  a.invd = ptr<float>(ws, li.invd32);
  a.acc = ptr<float>(ws, li.acc32);
  a.phi2 = li.phi2_32 ? ptr<float>(ws, li.phi2_32) : nullptr;
  a.onepass = li.onepass32 ? 1 : 0;
  a.fuseops = li.fuse_ops && li.phi2_32 ? 1 : 0;
  a.mx = li.m[0];
  a.my = li.m[1];
  a.mz = li.m[2];
  a.P = li.box.P;
  a.S = li.box.S;
  return a;
}
namespace {

template <typename T>
LvlTable<T> make_table(const JmgPlan* p, void* ws);
template <>
LvlTable<double> make_table<double>(const JmgPlan* p, void* ws) {
  LvlTable<double> t;
  memset(&t, 0, sizeof(t));
  for (int l = 0; l < p->used; ++l) t.l[l] = lvl64(p, ws, l);
  return t;
}
template <>
LvlTable<float> make_table<float>(const JmgPlan* p, void* ws) {
  LvlTable<float> t;
  memset(&t, 0, sizeof(t));
  for (int l = 0; l < p->used; ++l) t.l[l] = lvl32(p, ws, l);
  return t;
}

}  // namespace
CycleParams jmg::cycle_params(const JmgPlan* p, bool off_diag) {
  CycleParams cp;
  cp.last_level = p->levels - 2;
  cp.nu1 = p->cfg.nu1 > 0 ? p->cfg.nu1 : 0;
  cp.nu2 = p->cfg.nu2 > 0 ? p->cfg.nu2 : 0;
  cp.gamma = p->cfg.gamma > 0 ? p->cfg.gamma : 0;
  // 2D: the (even,even) points need prolongation if nu2 <= 0 or with D_xy
  // (solver_2d.py:665); 3D: the bilinear points if nu2 <= 0 (solver_3d.py:671)
  cp.diag = (p->cfg.nu2 <= 0 || off_diag) ? 1 : 0;
  return cp;
}
namespace {

// multigrid_cycle, solver_2d.py:582-614, emitted as launches on stream s. With a
// non-null `count`, nothing is launched and the number of kernel launches is added.
// Option of the outermost call of a cycle (level 0 only): start the first sweep from a
// zero guess without reading phi (a refinement step's correction).
struct EmitTop {
  bool zero_first = false;
};

// multigrid_cycle, solver_2d.py:582-614, emitted as launches on stream s. With a
// non-null `count`, nothing is launched and the number of kernel launches is added.
// zero_phi: phi of this level is zero on entry (the first visit after the restriction
// above zeroed it), so a fused pre-sweep need not read it.
template <typename T>
void emit_cycle(const JmgPlan* p, LvlTable<T>& tab, const LvlTable<T>* dtab, const CycleParams& cp, int lev,
                bool fcycle, bool skip_pre, cudaStream_t s, long long* count = nullptr,
                const EmitTop* top = nullptr, bool zero_phi = false, LoopState* st = nullptr) {
  const int dim = p->dim;
  // 2D: this level and everything below it in one cooperative launch (mg_mid2d.cu)
  const size_t mid_smem = sizeof(T) == 8 ? p->mid_smem64 : p->mid_smem32;
  if (p->mid_now && lev == p->mid_start && mid_smem && !skip_pre && (count || st)) {
    if (count) {
      *count += 1;
      return;
    }
    MidOps ops;
    if (mid_ops(cp, p->coarse_start, lev, fcycle, zero_phi, &ops)) {
      launch_mid2d<T>(dtab, st, cp, p->coarse_start, ops, mid_smem, p->mid_blocks, p->mid_stall, s);
      return;
    }
  }
  // Fused operator pairs on a grid-wide 2D level (mg_fusedops2d.cu): the last pre-sweep
  // with the restriction, the prolongation with the first post-sweep; each writes the
  // level's second buffer and swaps, so a visit swaps twice.
  const bool fuse = lev < p->coarse_start && lev != cp.last_level && tab.l[lev].fuseops && !tab.l[lev].xll &&
                    !skip_pre && cp.nu1 >= 1 && cp.nu2 >= 1;
  // One-pass sweeps write the level's second buffer and swap; an even number of them per
  // visit leaves phi where the visit found it (the restriction, the prolongation and the
  // caller's tables see the current buffer). An odd remainder runs as colour passes.
  const int nsweeps = lev == cp.last_level ? cp.nu1 + cp.nu2
                                           : (skip_pre ? 0 : cp.nu1) + cp.nu2 - (fuse ? 2 : 0);
  int fused_left = tab.l[lev].onepass ? nsweeps - nsweeps % 2 : 0;
  auto sweep = [&](bool first) {
    const bool zero = top && top->zero_first && first;
    if (fused_left > 0) {
      --fused_left;
      if (count) *count += 1;
      else launch_sweep_onepass<T>(dim, tab.l[lev], zero, s);
      return;
    }
    if (count) *count += dim == 2 && tab.l[lev].xll ? 4 : 2;  // colour (sub-lattice) passes
    else launch_sweep<T>(dim, tab.l[lev], s, zero);
  };
  if (lev >= p->coarse_start) {
    if (count) *count += 1;
    else if (p->cluster_ranks)
      launch_coarse_cluster<T>(dim, dtab, p->cluster, cp, fcycle ? 1 : 0, skip_pre ? 1 : 0,
                               sizeof(T) == 8 ? p->cluster_smem64 : p->cluster_smem32, s);
    else if (sizeof(T) == 4 && p->coarse_smem32)
      launch_coarse_smem32(reinterpret_cast<const LvlTable<float>*>(dtab), cp, lev, fcycle ? 1 : 0,
                           skip_pre ? 1 : 0, p->coarse_smem32, s);
    else if (lev == p->coarse_start && (sizeof(T) == 8 ? p->coarse_staged64 : p->coarse_staged32))
      launch_coarse_staged<T>(dim, dtab, cp, lev, fcycle ? 1 : 0, skip_pre ? 1 : 0,
                              sizeof(T) == 8 ? p->coarse_staged64 : p->coarse_staged32, p->coarse_threads, s);
    else launch_coarse_cycle<T>(dim, dtab, cp, lev, fcycle ? 1 : 0, skip_pre ? 1 : 0, s);
    return;
  }
  if (lev == cp.last_level) {
    for (int k = 0; k < cp.nu1 + cp.nu2; ++k) sweep(k == 0);
    return;
  }
  if (!skip_pre)
    for (int k = 0; k < cp.nu1 - (fuse ? 1 : 0); ++k) sweep(k == 0);
  if (count) *count += 1;
  else if (fuse)
    launch_smooth_restrict<T>(dim, tab.l[lev], tab.l[lev + 1], cp.nu1 == 1 && ((top && top->zero_first) || zero_phi),
                              s);
  else launch_restrict<T>(dim, tab.l[lev], tab.l[lev + 1], s);
  bool first = true;  // phi of level lev + 1 is zero until its first visit
  if (fcycle)
    for (int g = 0; g < cp.gamma; ++g) {
      emit_cycle<T>(p, tab, dtab, cp, lev + 1, true, false, s, count, nullptr, first, st);
      first = false;
    }
  for (int g = 0; g < cp.gamma; ++g) {
    emit_cycle<T>(p, tab, dtab, cp, lev + 1, false, false, s, count, nullptr, first, st);
    first = false;
  }
  if (count) *count += 1;
  else if (fuse) launch_prolong_smooth<T>(dim, tab.l[lev], tab.l[lev + 1], s);
  else launch_prolong<T>(dim, tab.l[lev], tab.l[lev + 1], cp.diag, s);
  for (int k = 0; k < cp.nu2 - (fuse ? 1 : 0); ++k) sweep(false);
}

// Whether the mixed-precision refinement step can use the short form: the FP32 cycle
// starts with a sweep at level 0 from a zero guess (no zeroing pass), and one tiled FP64
// kernel gives both the stopping test's residual and the next step's FP32 right-hand side.
bool mixed_fused(const JmgPlan* p) {
  return !p->fcg && !p->off_diag && p->mixed && p->dim == 2 && p->cfg.stop == JMG_STOP_RESIDUAL && !p->cfg.fixed && p->coarse_start > 0 &&
         p->cfg.nu1 >= 1 && p->cfg.nu2 >= 1;
}

// Mixed precision with the residual stop in any other case (3D, small grids, nu = 0):
// one FP64 pass computes the residual norm and the FP32 right-hand side together.
bool mixed_resid(const JmgPlan* p) {
  return !p->fcg && p->mixed && !mixed_fused(p) && p->cfg.stop == JMG_STOP_RESIDUAL && !p->cfg.fixed;
}

int loop_mode(const JmgPlan* p) {
  if (p->cfg.fixed) return 2;
  return p->cfg.stop == JMG_STOP_RESIDUAL ? 1 : 0;
}

// FCG step: z = cycle(rho) from z = 0 (FP32 inside refinement, or FP64), then the FCG
// update (mg_krylov.cu) and the loop test on ||rho||.
void emit_fcg_body(const JmgPlan* p, void* ws, unsigned long long handle, cudaStream_t s) {
  LoopState* st = ptr<LoopState>(ws, p->off_state);
  Lvl<double> l0 = lvl64(p, ws, 0);
  CycleParams cp = cycle_params(p, p->off_diag);
  double* fp = ptr<double>(ws, p->off_fcg_parts);
  const int np = fcg_num_parts();
  const int inner = p->cfg.inner_cycles > 0 ? p->cfg.inner_cycles : 1;
  // the first sweep may start from a zero guess without reading phi when level 0 runs its
  // own sweeps; otherwise the correction is zeroed first
  const bool zero_first = p->coarse_start > 0 && p->cfg.nu1 >= 1;
  if (p->mixed) {
    LvlTable<float> t32 = make_table<float>(p, ws);
    if (!zero_first) cudaMemsetAsync(t32.l[0].phi, 0, p->lv[0].elems * 4, s);
    for (int k = 0; k < inner; ++k) {
      EmitTop top;
      top.zero_first = zero_first && k == 0;
      emit_cycle<float>(p, t32, ptr<LvlTable<float>>(ws, p->off_tab32), cp, 0, p->cfg.fcycle != 0, false, s,
                        nullptr, &top, false, st);
    }
    launch_fcg32_iter(p->dim, l0, t32.l[0], t32.l[0].phi, ptr<float>(ws, p->off_d), ptr<float>(ws, p->off_q),
                      t32.l[0].rhs, fp, fp + 2 * np, fp + 4 * np, s);
  } else {
    LvlTable<double> tz = make_table<double>(p, ws);
    tz.l[0].phi = ptr<double>(ws, p->off_z64);
    tz.l[0].rhs = ptr<double>(ws, p->off_rho);
    if (!zero_first) cudaMemsetAsync(tz.l[0].phi, 0, p->lv[0].elems * 8, s);
    for (int k = 0; k < inner; ++k) {
      EmitTop top;
      top.zero_first = zero_first && k == 0;
      emit_cycle<double>(p, tz, ptr<LvlTable<double>>(ws, p->off_tab64z), cp, 0, p->cfg.fcycle != 0, false, s,
                         nullptr, &top, false, st);
    }
    launch_fcg_iter<double>(p->dim, l0, tz.l[0].phi, ptr<double>(ws, p->off_d), ptr<double>(ws, p->off_q),
                            ptr<double>(ws, p->off_rho), nullptr, fp, fp + 2 * np, fp + 4 * np, s);
  }
  launch_loop_step(st, fp + 4 * np, fcg_parts_used(p->dim, l0), loop_mode(p), p->cfg.epsilon, p->cfg.rtol,
                   p->cfg.max_iters_outer, handle, s);
}

// body of one loop iteration (captured into the WHILE node's body graph)
void emit_body(const JmgPlan* p, void* ws, unsigned long long handle, cudaStream_t s) {
  const int mode = loop_mode(p);
  LoopState* st = ptr<LoopState>(ws, p->off_state);
  double* parts = ptr<double>(ws, p->off_parts);
  Lvl<double> l0 = lvl64(p, ws, 0);
  CycleParams cp = cycle_params(p, p->off_diag);
  int nparts = p->nparts;
  if (p->fcg) {
    emit_fcg_body(p, ws, handle, s);
    return;
  }
  if (!p->mixed) {
    LvlTable<double> tab = make_table<double>(p, ws);
    emit_cycle<double>(p, tab, ptr<LvlTable<double>>(ws, p->off_tab64), cp, 0, p->cfg.fcycle != 0,
                       p->cfg.skip_pre != 0, s, nullptr, nullptr, false, st);
  } else if (mixed_fused(p)) {
    // FP64 iterative refinement around FP32 cycles. r32 = float(rhs - L_h phi) is already
    // in place (prologue or previous step). FP32 cycles solve L_h e = r from e = 0; the
    // last sweep adds e to phi (FP64); then the FP64 residual for the next step and the
    // stopping test.
    LvlTable<float> t32 = make_table<float>(p, ws);
    const int inner = p->cfg.inner_cycles > 0 ? p->cfg.inner_cycles : 1;
    for (int k = 0; k < inner; ++k) {
      EmitTop top;
      top.zero_first = k == 0;
      emit_cycle<float>(p, t32, ptr<LvlTable<float>>(ws, p->off_tab32), cp, 0, p->cfg.fcycle != 0, false, s,
                        nullptr, &top, false, st);
    }
    launch_add_correction(p->dim, l0, t32.l[0].phi, s);
    launch_residual_f32_2d(l0, t32.l[0].rhs, parts, s);
    nparts = residual_f32_parts2d(l0.mx, l0.my);
  } else {
    // FP64 iterative refinement around FP32 cycles: r = rhs - L_h phi (FP64), solve
    // L_h e = r with FP32 cycles from e = 0, phi += e (FP64). With the residual stop, r32
    // comes from the previous step's residual pass (or the prologue).
    LvlTable<float> t32 = make_table<float>(p, ws);
    if (!mixed_resid(p)) launch_residual_to_f32(p->dim, l0, t32.l[0].rhs, s);
    launch_zero_f32(p->lv[0].box, t32.l[0].phi, s);
    const int inner = p->cfg.inner_cycles > 0 ? p->cfg.inner_cycles : 1;
    for (int k = 0; k < inner; ++k)
      emit_cycle<float>(p, t32, ptr<LvlTable<float>>(ws, p->off_tab32), cp, 0, p->cfg.fcycle != 0, false, s,
                        nullptr, nullptr, false, st);
    launch_add_correction(p->dim, l0, t32.l[0].phi, s);
    if (mixed_resid(p)) launch_residual_partials<double>(p->dim, l0, l0.phi, parts, p->nparts, s, t32.l[0].rhs);
  }
  if (mode == 0) launch_distance_snapshot(p->lv[0].box, ptr<double>(ws, p->off_phi_old), l0.phi, st, s);
  if (mode == 1 && !p->mixed) launch_residual_partials<double>(p->dim, l0, l0.phi, parts, p->nparts, s);
  launch_loop_step(st, parts, nparts, mode, p->cfg.epsilon, p->cfg.rtol, p->cfg.max_iters_outer, handle, s);
}

// loop prologue: initial residual (residual stop) and loop init
void emit_prologue(const JmgPlan* p, void* ws, unsigned long long handle, cudaStream_t s) {
  const int mode = loop_mode(p);
  LoopState* st = ptr<LoopState>(ws, p->off_state);
  double* parts = ptr<double>(ws, p->off_parts);
  Lvl<double> l0 = lvl64(p, ws, 0);
  int nparts = p->nparts;
  if (p->fcg) {
    double* fp = ptr<double>(ws, p->off_fcg_parts);
    if (p->mixed)
      launch_fcg32_init(p->dim, l0, lvl32(p, ws, 0).rhs, ptr<float>(ws, p->off_d), ptr<float>(ws, p->off_q), fp, s);
    else
      launch_fcg_init(p->dim, l0, ptr<double>(ws, p->off_rho), ptr<double>(ws, p->off_d), ptr<double>(ws, p->off_q),
                      nullptr, fp, s);
    launch_loop_init(st, fp, fcg_parts_used(p->dim, l0), mode, p->cfg.rtol, p->cfg.max_iters_outer, handle, s);
    return;
  }
  if (mixed_fused(p)) {
    launch_residual_f32_2d(l0, lvl32(p, ws, 0).rhs, parts, s);
    nparts = residual_f32_parts2d(l0.mx, l0.my);
  } else if (mixed_resid(p)) {
    launch_residual_partials<double>(p->dim, l0, l0.phi, parts, p->nparts, s, lvl32(p, ws, 0).rhs);
  } else if (mode == 1) {
    launch_residual_partials<double>(p->dim, l0, l0.phi, parts, p->nparts, s);
  }
  launch_loop_init(st, parts, nparts, mode, p->cfg.rtol, p->cfg.max_iters_outer, handle, s);
}

// Counting emits no launch and reads no array: tables over this placeholder workspace
// address only tell which arrays a level has (second phi buffers, D_xy couplings).
void* const kCountBase = reinterpret_cast<void*>(static_cast<uintptr_t>(kAlign));

long long body_launches(const JmgPlan* p) {
  long long n = 0;
  CycleParams cp = cycle_params(p, p->off_diag);
  if (p->fcg) {
    const int inner = p->cfg.inner_cycles > 0 ? p->cfg.inner_cycles : 1;
    const bool zero_first = p->coarse_start > 0 && p->cfg.nu1 >= 1;
    if (p->mixed) {
      LvlTable<float> t = make_table<float>(p, kCountBase);
      for (int k = 0; k < inner; ++k) emit_cycle<float>(p, t, nullptr, cp, 0, p->cfg.fcycle != 0, false, nullptr, &n);
    } else {
      LvlTable<double> t = make_table<double>(p, kCountBase);
      for (int k = 0; k < inner; ++k) emit_cycle<double>(p, t, nullptr, cp, 0, p->cfg.fcycle != 0, false, nullptr, &n);
    }
    return n + (p->mixed ? 4 : 3) + 1 + (zero_first ? 0 : 1);  // FCG update, loop step (+ memset node)
  }
  if (!p->mixed) {
    LvlTable<double> t = make_table<double>(p, kCountBase);
    emit_cycle<double>(p, t, nullptr, cp, 0, p->cfg.fcycle != 0, p->cfg.skip_pre != 0, nullptr, &n);
  } else {
    LvlTable<float> t = make_table<float>(p, kCountBase);
    const int inner = p->cfg.inner_cycles > 0 ? p->cfg.inner_cycles : 1;
    for (int k = 0; k < inner; ++k) emit_cycle<float>(p, t, nullptr, cp, 0, p->cfg.fcycle != 0, false, nullptr, &n);
    n += mixed_fused(p) ? 2 : (mixed_resid(p) ? 3 : 3 + (loop_mode(p) == 0));
  }
  const int mode = loop_mode(p);
  if (!p->mixed && (mode == 0 || mode == 1)) n += 1;  // distance or residual partials
  n += 1;                                             // loop step
  return n;
}

int capture_graph(JmgPlan* p, void* ws, cudaGraphExec_t* out) {
  for (const JmgPlan::GraphSlot& g : p->graphs)
    if (g.ws == ws && g.mid == p->mid_now) {
      *out = g.exec;
      return JMG_OK;
    }
  if ((int)p->graphs.size() >= JmgPlan::kMaxGraphs) {
    // an exec still in flight is freed by the runtime once it completes
    cudaGraphExecDestroy(p->graphs.front().exec);
    p->graphs.erase(p->graphs.begin());
  }
  if (!p->cap) JMG_CUDA(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
  cudaGraph_t graph;
  JMG_CUDA(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle handle;
  JMG_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 0, 0));
  // prologue: initial residual (residual stop) and loop init, then the WHILE node
  JMG_CUDA(cudaStreamBeginCaptureToGraph(p->cap, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  emit_prologue(p, ws, handle, p->cap);
  cudaStreamCaptureStatus cst;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  JMG_CUDA(cudaStreamGetCaptureInfo(p->cap, &cst, nullptr, nullptr, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cparams = {cudaGraphNodeTypeConditional};
  cparams.conditional.handle = handle;
  cparams.conditional.type = cudaGraphCondTypeWhile;
  cparams.conditional.size = 1;
  cudaGraphNode_t cnode;
  JMG_CUDA(cudaGraphAddNode(&cnode, graph, deps, nullptr, ndeps, &cparams));
  JMG_CUDA(cudaStreamUpdateCaptureDependencies(p->cap, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  JMG_CUDA(cudaStreamEndCapture(p->cap, &graph));
  cudaGraph_t body = cparams.conditional.phGraph_out[0];
  JMG_CUDA(cudaStreamBeginCaptureToGraph(p->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  emit_body(p, ws, (unsigned long long)handle, p->cap);
  JMG_CUDA(cudaGetLastError());
  cudaGraph_t body_out = body;
  JMG_CUDA(cudaStreamEndCapture(p->cap, &body_out));
  cudaGraphExec_t exec;
  JMG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  cudaGraphDestroy(graph);
  p->graphs.push_back({ws, exec, p->mid_now});
  *out = exec;
  return JMG_OK;
}

// The loop graph; if capturing or instantiating it with the cooperative middle-level
// kernel fails (a runtime that does not take cooperative kernel nodes in conditional
// graphs), the plan drops that kernel and captures the plain launches instead.
int build_graph(JmgPlan* p, void* ws, cudaGraphExec_t* out) {
  const int rc = capture_graph(p, ws, out);
  if (rc == JMG_OK || !p->mid_now) return rc;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (p->cap && cudaStreamIsCapturing(p->cap, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(p->cap, &g);
    if (g) cudaGraphDestroy(g);
  }
  cudaGetLastError();
  p->mid_start = -1;
  p->mid_smem32 = p->mid_smem64 = 0;
  p->mid_now = false;
  return capture_graph(p, ws, out);
}

HierInputs hier_inputs(const JmgPlan* p, const JmgCoeffs* c) {
  HierInputs in;
  in.lam = c->lam;
  in.lam_scalar = c->lam_scalar;
  in.scalar_lam = c->lam == nullptr;
  int nscalar = 0;
  for (int a = 0; a < 3; ++a) {
    in.D[a] = a < p->dim ? c->D[a] : nullptr;
    in.D_scalar[a] = a < p->dim ? c->D_scalar[a] : 0.0;
    if (a < p->dim && c->D[a] == nullptr) ++nscalar;
  }
  in.scalar_D = nscalar == p->dim;
  in.Dxy = (p->off_diag && !in.scalar_D) ? c->D_xy : nullptr;
  return in;
}

}  // namespace
int jmg::check_coeffs(const JmgPlan* p, const JmgCoeffs* c) {
  if (!c) return set_err(JMG_ERR_VALUE, "coeffs must not be NULL");
  int nscalar = 0;
  for (int a = 0; a < p->dim; ++a)
    if (c->D[a] == nullptr) ++nscalar;
  if (nscalar != 0 && nscalar != p->dim)
    return set_err(JMG_ERR_VALUE, "Shape mismatch: the D components must be all scalars or all arrays.");
  if (c->D_xy && p->dim == 3) return set_err(JMG_ERR_VALUE, "D_xy is a 2D argument");
  // D_xy takes part only with array D (solver_2d.py:333: off_diag needs spatial D)
  const bool uses = c->D_xy && nscalar == 0;
  if (uses && !p->off_diag)
    return set_err(JMG_ERR_VALUE, "D_xy with array D needs a plan created with cfg.off_diag = 1");
  if (!uses && p->off_diag)
    return set_err(JMG_ERR_VALUE, "a plan created with cfg.off_diag = 1 needs D_xy and array D");
  return JMG_OK;
}
namespace {

}  // namespace
int jmg::check_ws(const JmgPlan* p, void* ws, size_t bytes) {
  if (!p) return set_err(JMG_ERR_VALUE, "plan must not be NULL");
  if (!ws || bytes < p->ws_bytes)
    return set_err(JMG_ERR_WORKSPACE, "workspace too small: %zu bytes given, %zu needed", bytes, p->ws_bytes);
  if (reinterpret_cast<uintptr_t>(ws) % kAlign != 0)
    return set_err(JMG_ERR_WORKSPACE, "workspace must be %zu-byte aligned", kAlign);
  return JMG_OK;
}
namespace {

}  // namespace
int jmg::build_hierarchy(JmgPlan* p, const JmgCoeffs* c, void* ws, cudaStream_t s) {
  const HierInputs in = hier_inputs(p, c);

  const Box b0 = p->lv[0].box;
  for (int l = 0; l < p->used; ++l) {
    const LevelInfo& li = p->lv[l];
    double sq[3], idl[3];
    for (int a = 0; a < 3; ++a) {
      const double id = a < p->dim ? p->grid.idel[a] * std::pow(0.5, l) : 0.0;  // solver_2d.py:323
      idl[a] = id;
      sq[a] = id * id;                                                         // solver_2d.py:395
    }
    double* dcur[3] = {nullptr, nullptr, nullptr};
    const double* dprev[3] = {nullptr, nullptr, nullptr};
    Box bprev = b0;
    if (p->dim == 3 && l >= 1) {
      for (int a = 0; a < 3; ++a) dcur[a] = ptr<double>(ws, li.d[a]);
      if (l >= 2) {
        for (int a = 0; a < 3; ++a) dprev[a] = ptr<double>(ws, p->lv[l - 1].d[a]);
        bprev = p->lv[l - 1].box;
      }
    }
    launch_hierarchy_level(p->dim, l, lvl64(p, ws, l), li.box, b0, in, idl, sq, dcur, dprev, bprev, s);
  }
  if (p->mixed) {
    for (int l = 0; l < p->used; ++l) {
      const LevelInfo& li = p->lv[l];
      Lvl<double> a = lvl64(p, ws, l);
      Lvl<float> f = lvl32(p, ws, l);
      launch_convert_f32(li.box, a.wx, f.wx, s);
      launch_convert_f32(li.box, a.wy, f.wy, s);
      if (p->dim == 3) launch_convert_f32(li.box, a.wz, f.wz, s);
      launch_convert_f32(li.box, a.invd, f.invd, s);
      launch_convert_f32(li.box, a.acc, f.acc, s);
      if (p->off_diag) {
        launch_convert_f32(li.box, a.xll, f.xll, s);
        launch_convert_f32(li.box, a.xrl, f.xrl, s);
        launch_convert_f32(li.box, a.xlr, f.xlr, s);
        launch_convert_f32(li.box, a.xrr, f.xrr, s);
      }
    }
  }
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}
namespace {

__global__ void k_write_i64(long long* out, long long v) { *out = v; }

}  // namespace

int jmg::set_error_message(int code, const char* msg) { return set_err(code, "%s", msg); }

int jmg::block_coarse_level(const JmgPlan* p) { return block_coarse_start(p); }

// JMG_PDL=0 turns programmatic dependent launch off (read once per process)
bool jmg::pdl_enabled() {
  static const bool on = [] {
    const char* e = getenv("JMG_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------

// nsweeps sweeps of one level as a solve runs them: one-pass sweeps in pairs where the
// level has a second buffer (phi ends in the buffer it started in), colour passes else
template <typename T>
static void smooth_like_solve(const JmgPlan* p, Lvl<T>& a, int nsweeps, cudaStream_t s) {
  const int fused = a.onepass ? nsweeps - nsweeps % 2 : 0;
  for (int k = 0; k < fused; ++k) launch_sweep_onepass<T>(p->dim, a, false, s);
  for (int k = fused; k < nsweeps; ++k) launch_sweep<T>(p->dim, a, s);
}

extern "C" {

void jmg_config_default(JmgConfig* c) {
  memset(c, 0, sizeof(*c));
  c->fixed = 0;
  c->gamma = 1;
  c->fcycle = 0;
  c->skip_pre = 0;
  c->nu1 = 1;
  c->nu2 = 1;
  c->max_iters_outer = 2147483647LL;
  c->max_iters_inner = 2147483647LL;
  c->epsilon = 1e-12;
  c->stop = JMG_STOP_DISTANCE;
  c->rtol = 1e-10;
  c->precision = JMG_PREC_FP64;
  c->inner_cycles = 1;
  c->outer = JMG_OUTER_RICHARDSON;
}

int jmg_plan_create(JmgPlan** out, const JmgGrid* grid, const JmgConfig* cfg) {
  if (!out || !grid || !cfg) return set_err(JMG_ERR_VALUE, "NULL argument");
  *out = nullptr;
  JmgPlan* p = new JmgPlan();
  p->grid = *grid;
  p->cfg = *cfg;
  const int rc = validate_and_layout(p);
  if (rc != JMG_OK) {
    delete p;
    return rc;
  }
  *out = p;
  g_last_error.clear();
  return JMG_OK;
}

int jmg_plan_destroy(JmgPlan* p) {
  if (!p) return JMG_OK;
  for (const JmgPlan::GraphSlot& g : p->graphs) cudaGraphExecDestroy(g.exec);
  if (p->vjp_exec) cudaGraphExecDestroy(p->vjp_exec);
  if (p->cap) cudaStreamDestroy(p->cap);
  for (cudaStream_t ls : p->lane_streams) cudaStreamDestroy(ls);
  for (cudaEvent_t ev : p->lane_events) cudaEventDestroy(ev);
  if (p->fork_event) cudaEventDestroy(p->fork_event);
  delete p;
  return JMG_OK;
}

size_t jmg_plan_workspace_bytes(const JmgPlan* p) { return p ? p->ws_bytes : 0; }
int jmg_plan_levels(const JmgPlan* p) { return p ? p->levels : 0; }

int jmg_build_hierarchy(JmgPlan* p, const JmgCoeffs* c, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc) return rc;
  if ((rc = check_coeffs(p, c))) return rc;
  return build_hierarchy(p, c, ws, (cudaStream_t)stream);
}

int jmg_solve(JmgPlan* p, const double* phi0, const double* rhs, const JmgCoeffs* c, double* phi_out,
              int64_t* count_out, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc) return rc;
  if ((rc = check_coeffs(p, c))) return rc;
  if (!phi0 || !rhs || !phi_out) return set_err(JMG_ERR_VALUE, "phi0, rhs and phi_out must not be NULL");
  if ((rc = coarse_setup(p))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const Box b0 = p->lv[0].box;
  Lvl<double> l0 = lvl64(p, ws, 0);
  LoopState* st = ptr<LoopState>(ws, p->off_state);
  double* parts = ptr<double>(ws, p->off_parts);
  double* phi_old = ptr<double>(ws, p->off_phi_old);
  const int mode = loop_mode(p);
  // 1. inputs; phi_old keeps phi0 with its frame (the first distance sees it, solver_2d.py:471)
  launch_copy_in(b0, phi0, l0.phi, 1, s);
  launch_copy_in(b0, phi0, phi_old, 0, s);
  launch_copy_in(b0, rhs, l0.rhs, 1, s);
  // 2. coefficients, and the level tables the single-block coarse kernel reads
  if ((rc = build_hierarchy(p, c, ws, s))) return rc;
  launch_store_table<double>(make_table<double>(p, ws), ptr<LvlTable<double>>(ws, p->off_tab64), s);
  if (p->fcg) {
    // zero frames of the FCG vectors (their kernels write interiors only)
    const size_t b8 = p->lv[0].elems * 8, bv = p->lv[0].elems * (p->mixed ? 4 : 8);
    if (!p->mixed) JMG_CUDA(cudaMemsetAsync(ptr<char>(ws, p->off_rho), 0, b8, s));
    JMG_CUDA(cudaMemsetAsync(ptr<char>(ws, p->off_d), 0, bv, s));
    JMG_CUDA(cudaMemsetAsync(ptr<char>(ws, p->off_q), 0, bv, s));
    if (!p->mixed) {
      JMG_CUDA(cudaMemsetAsync(ptr<char>(ws, p->off_z64), 0, b8, s));
      LvlTable<double> tz = make_table<double>(p, ws);
      tz.l[0].phi = ptr<double>(ws, p->off_z64);
      tz.l[0].rhs = ptr<double>(ws, p->off_rho);
      launch_store_table<double>(tz, ptr<LvlTable<double>>(ws, p->off_tab64z), s);
    }
  }
  // second phi buffers: their frames must read zero (sweeps write interiors only)
  for (int l = 0; l < p->used; ++l) {
    const LevelInfo& li = p->lv[l];
    if (li.phi2) JMG_CUDA(cudaMemsetAsync(ptr<char>(ws, li.phi2), 0, li.elems * 8, s));
    if (li.phi2_32) JMG_CUDA(cudaMemsetAsync(ptr<char>(ws, li.phi2_32), 0, li.elems * 4, s));
  }
  if (p->mixed) {
    launch_store_table<float>(make_table<float>(p, ws), ptr<LvlTable<float>>(ws, p->off_tab32), s);
    // zero frames of the FP32 correction and residual of level 0 (kernels write only interiors)
    launch_zero_f32(b0, lvl32(p, ws, 0).phi, s);
    launch_zero_f32(b0, lvl32(p, ws, 0).rhs, s);
  }
  if (mode == 1) {
    launch_residual_partials<double>(p->dim, l0, nullptr, parts, p->nparts, s);
    launch_rhs_norm(st, parts, p->nparts, s);
  }
  // 3. skip_pre: pre-smoothing once, before the loop (solver_2d.py:457-459)
  const int nu1 = p->cfg.nu1 > 0 ? p->cfg.nu1 : 0;
  const bool presmoothed = p->cfg.skip_pre && nu1 > 0;
  if (presmoothed) {
    Lvl<double> cur = l0;
    for (int k = 0; k < nu1; ++k) launch_sweep<double>(p->dim, cur, s);
    launch_distance_snapshot(b0, phi_old, l0.phi, st, s);  // phi_old <- smoothed phi
  }
  // 4. the loop (the cooperative middle-level kernel only outside the lanes of a batch)
  p->mid_now = p->mid_start >= 0 && !p->in_batch;
  const bool runs = p->cfg.max_iters_outer > 0;
  // the loop's prologue clears the fault flag jmg_solve_check reads; without a loop, here
  if (!runs) JMG_CUDA(cudaMemsetAsync(&st->fault, 0, sizeof(int), s));
  if (runs && !p->host_loop) {
    cudaGraphExec_t exec = nullptr;
    if ((rc = build_graph(p, ws, &exec))) return rc;
    JMG_CUDA(cudaGraphLaunch(exec, s));
  } else if (runs) {
    emit_prologue(p, ws, 0, s);
    for (;;) {
      int go = 0;
      JMG_CUDA(cudaMemcpyAsync(&go, &st->go, sizeof(int), cudaMemcpyDeviceToHost, s));
      JMG_CUDA(cudaStreamSynchronize(s));
      if (!go) break;
      emit_body(p, ws, 0, s);
    }
  }
  // 5. outputs. With no cycle and no smoothing the reference returns phi0 untouched.
  if (runs || presmoothed)
    launch_copy_out(b0, l0.phi, phi_out, s);
  else if (phi_out != phi0)
    JMG_CUDA(cudaMemcpyAsync(phi_out, phi0, (size_t)b0.nx * b0.ny * b0.nz * 8, cudaMemcpyDeviceToDevice, s));
  if (count_out) {
    if (p->cfg.fixed || !runs)
      k_write_i64<<<1, 1, 0, s>>>((long long*)count_out, p->cfg.fixed ? p->cfg.max_iters_outer : 0);
    else
      launch_count_out(st, (long long*)count_out, s);
  }
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

static int solve_oneshot(int dim, const JmgGrid* grid, const JmgConfig* cfg, const double* phi0, const double* rhs,
                         const JmgCoeffs* c, double* phi_out, int64_t* count_out, void* ws, size_t bytes,
                         jmg_stream_t stream) {
  if (!grid || grid->ndim != dim) return set_err(JMG_ERR_VALUE, "grid->ndim must be %d", dim);
  if (!cfg || !c) return set_err(JMG_ERR_VALUE, "NULL argument");
  // the one-shot form sets off_diag itself: D_xy with array D selects the 9-point stencil
  JmgConfig cf = *cfg;
  cf.off_diag = dim == 2 && c->D_xy && c->D[0] && c->D[1] ? 1 : 0;
  JmgPlan* p = nullptr;
  int rc = jmg_plan_create(&p, grid, &cf);
  if (rc) return rc;
  rc = jmg_solve(p, phi0, rhs, c, phi_out, count_out, ws, bytes, stream);
  if (rc == JMG_OK && !p->graphs.empty()) {
    // the graph exec is destroyed with the plan: wait for the launch to finish first
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) rc = set_err(JMG_ERR_CUDA, "cudaStreamSynchronize failed: %s", cudaGetErrorString(e));
  }
  jmg_plan_destroy(p);
  return rc;
}

int jmg_solve2d_f64(const JmgGrid* grid, const JmgConfig* cfg, const double* phi0, const double* rhs,
                    const JmgCoeffs* c, double* phi_out, int64_t* count_out, void* ws, size_t bytes,
                    jmg_stream_t stream) {
  return solve_oneshot(2, grid, cfg, phi0, rhs, c, phi_out, count_out, ws, bytes, stream);
}

int jmg_solve3d_f64(const JmgGrid* grid, const JmgConfig* cfg, const double* phi0, const double* rhs,
                    const JmgCoeffs* c, double* phi_out, int64_t* count_out, void* ws, size_t bytes,
                    jmg_stream_t stream) {
  return solve_oneshot(3, grid, cfg, phi0, rhs, c, phi_out, count_out, ws, bytes, stream);
}

static int level_check(const JmgPlan* p, int level, bool needs_coarse) {
  if (level < 0 || level >= p->used || (needs_coarse && level + 1 >= p->used))
    return set_err(JMG_ERR_VALUE, "level %d out of range", level);
  return JMG_OK;
}

int jmg_op_sweep(JmgPlan* p, int level, double* phi, const double* rhs, void* ws, size_t bytes,
                 jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, false))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Lvl<double> a = lvl64(p, ws, level);
  const Box b = p->lv[level].box;
  launch_copy_in(b, phi, a.phi, 1, s);  // the sweep starts with do_BCs (solver_2d.py:682)
  launch_copy_in(b, rhs, a.rhs, 0, s);
  launch_sweep<double>(p->dim, a, s);
  launch_copy_out(b, a.phi, phi, s);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_restrict(JmgPlan* p, int level, const double* phi, const double* rhs, double* rhs_c, void* ws,
                    size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, true))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Lvl<double> f = lvl64(p, ws, level), c = lvl64(p, ws, level + 1);
  const Box b = p->lv[level].box;
  launch_copy_in(b, phi, f.phi, 1, s);
  launch_copy_in(b, rhs, f.rhs, 0, s);
  launch_restrict<double>(p->dim, f, c, s);
  launch_copy_out(p->lv[level + 1].box, c.rhs, rhs_c, s);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_prolong(JmgPlan* p, int level, double* phi, const double* phi_c, void* ws, size_t bytes,
                   jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, true))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Lvl<double> f = lvl64(p, ws, level), c = lvl64(p, ws, level + 1);
  launch_copy_in(p->lv[level].box, phi, f.phi, 0, s);
  launch_copy_in(p->lv[level + 1].box, phi_c, c.phi, 0, s);
  launch_prolong<double>(p->dim, f, c, cycle_params(p, p->off_diag).diag, s);
  launch_copy_out(p->lv[level].box, f.phi, phi, s);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_residual(JmgPlan* p, int level, const double* phi, const double* rhs, double* d, void* ws,
                    size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, false))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Lvl<double> a = lvl64(p, ws, level);
  const Box b = p->lv[level].box;
  launch_copy_in(b, phi, a.phi, 1, s);
  launch_copy_in(b, rhs, a.rhs, 0, s);
  launch_dense_residual(p->dim, a, b, d, s);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_coeff(JmgPlan* p, int level, int which, double* out, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, false))) return rc;
  Lvl<double> a = lvl64(p, ws, level);
  const double* src = which == 0 ? a.acc : which == 1 ? a.wx : which == 2 ? a.wy : which == 3 ? a.wz : nullptr;
  if (!src) return set_err(JMG_ERR_VALUE, "no coefficient array %d in %dD", which, p->dim);
  launch_copy_coeff(p->lv[level].box, src, out, (cudaStream_t)stream);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_rel_residual(JmgPlan* p, const double* phi, const double* rhs, double* out, void* ws, size_t bytes,
                     jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Lvl<double> a = lvl64(p, ws, 0);
  const Box b = p->lv[0].box;
  LoopState* st = ptr<LoopState>(ws, p->off_state);
  double* parts = ptr<double>(ws, p->off_parts);
  launch_copy_in(b, phi, a.phi, 1, s);
  launch_copy_in(b, rhs, a.rhs, 1, s);
  launch_residual_partials<double>(p->dim, a, nullptr, parts, p->nparts, s);
  launch_rhs_norm(st, parts, p->nparts, s);
  launch_residual_partials<double>(p->dim, a, a.phi, parts, p->nparts, s);
  launch_rel_residual_out(st, parts, p->nparts, out, s);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_do_bcs(int ndim, const int32_t* shape, double* arr, jmg_stream_t stream) {
  if (ndim != 2 && ndim != 3) return set_err(JMG_ERR_VALUE, "ndim must be 2 or 3");
  launch_do_bcs_dense(ndim, shape, arr, (cudaStream_t)stream);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_plan_launch_counts(const JmgPlan* p, int64_t* per_solve_fixed, int64_t* per_cycle) {
  if (!p) return set_err(JMG_ERR_VALUE, "plan must not be NULL");
  // copy-ins (3), hierarchy (2 per level + FP32 conversions), rhs norm (2), loop init
  // (1-2), copy-out and count (2)
  long long fixed = 3 + 2LL * p->used + 2 + 2 + (p->mixed ? 4 : 1);
  if (p->mixed) fixed += (long long)p->used * (p->dim == 3 ? 5 : 4);
  if (loop_mode(p) == 1) fixed += 2 + 1;
  fixed += 1;
  if (p->cfg.skip_pre) fixed += 2LL * (p->cfg.nu1 > 0 ? p->cfg.nu1 : 0) + 1;
  if (per_solve_fixed) *per_solve_fixed = fixed;
  if (per_cycle) *per_cycle = body_launches(p);
  return JMG_OK;
}

int jmg_op_smooth_ws(JmgPlan* p, int level, int nsweeps, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, false))) return rc;
  Lvl<double> a = lvl64(p, ws, level);
  smooth_like_solve<double>(p, a, nsweeps, (cudaStream_t)stream);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_smooth32_ws(JmgPlan* p, int level, int nsweeps, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, false))) return rc;
  if (!p->mixed) return set_err(JMG_ERR_VALUE, "jmg_op_smooth32_ws needs a plan with precision mixed");
  Lvl<float> a = lvl32(p, ws, level);
  smooth_like_solve<float>(p, a, nsweeps, (cudaStream_t)stream);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_coarse_ws(JmgPlan* p, int fp32, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc) return rc;
  if (fp32 && !p->mixed) return set_err(JMG_ERR_VALUE, "jmg_op_coarse_ws(fp32=1) needs a plan with precision mixed");
  if ((rc = coarse_setup(p))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const CycleParams cp = cycle_params(p, p->off_diag);
  const int lev = p->coarse_start;
  if (fp32) {
    LvlTable<float> t = make_table<float>(p, ws);
    LvlTable<float>* dt = ptr<LvlTable<float>>(ws, p->off_tab32);
    launch_store_table<float>(t, dt, s);
    emit_cycle<float>(p, t, dt, cp, lev, false, false, s);
  } else {
    LvlTable<double> t = make_table<double>(p, ws);
    LvlTable<double>* dt = ptr<LvlTable<double>>(ws, p->off_tab64);
    launch_store_table<double>(t, dt, s);
    emit_cycle<double>(p, t, dt, cp, lev, false, false, s);
  }
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_op_fcg_residual_ws(JmgPlan* p, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc) return rc;
  if (!p->fcg || !p->mixed)
    return set_err(JMG_ERR_VALUE, "jmg_op_fcg_residual_ws needs a plan with outer fcg and precision mixed");
  // the kernel that ends every mixed FCG step (launch_fcg32_iter): rho = rhs - L x in FP64,
  // r32 = float(rho), partial sums of rho . rho
  launch_fcg32_init(p->dim, lvl64(p, ws, 0), lvl32(p, ws, 0).rhs, nullptr, nullptr,
                    ptr<double>(ws, p->off_fcg_parts) + 4 * fcg_num_parts(), (cudaStream_t)stream);
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_plan_coarse_start(const JmgPlan* p) { return p ? p->coarse_start : -1; }
int jmg_plan_mid_start(const JmgPlan* p) { return p && p->mid_start >= 0 && p->mid_now ? p->mid_start : -1; }

int jmg_plan_level_fused(const JmgPlan* p, int level, int fp32) {
  if (!p || level < 0 || level + 1 >= p->used) return 0;
  const LevelInfo& li = p->lv[level];
  return li.fuse_ops && (fp32 ? li.phi2_32 != 0 : li.phi2 != 0) ? 1 : 0;
}

int jmg_op_smooth_restrict_ws(JmgPlan* p, int level, int fp32, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc || (rc = level_check(p, level, true))) return rc;
  if (fp32 && !p->mixed) return set_err(JMG_ERR_VALUE, "jmg_op_smooth_restrict_ws(fp32=1) needs a plan with precision mixed");
  cudaStream_t s = (cudaStream_t)stream;
  const bool fused = jmg_plan_level_fused(p, level, fp32) != 0;
  if (fused && (rc = coarse_setup(p))) return rc;  // the fused kernels' attributes
  if (fp32) {
    Lvl<float> f = lvl32(p, ws, level), c = lvl32(p, ws, level + 1);
    if (fused) launch_smooth_restrict<float>(p->dim, f, c, false, s);
    else {
      launch_sweep<float>(p->dim, f, s);
      launch_restrict<float>(p->dim, f, c, s);
    }
  } else {
    Lvl<double> f = lvl64(p, ws, level), c = lvl64(p, ws, level + 1);
    if (fused) launch_smooth_restrict<double>(p->dim, f, c, false, s);
    else {
      launch_sweep<double>(p->dim, f, s);
      launch_restrict<double>(p->dim, f, c, s);
    }
  }
  JMG_CUDA(cudaGetLastError());
  return JMG_OK;
}

int jmg_plan_sweep_launches(const JmgPlan* p, int level, int fp32) {
  if (!p || level < 0 || level >= p->used) return 0;
  const LevelInfo& li = p->lv[level];
  if (fp32 ? li.onepass32 : li.onepass64) return 1;
  return p->off_diag ? 4 : 2;
}

int jmg_solve_check(JmgPlan* p, void* ws, size_t bytes, jmg_stream_t stream) {
  int rc = check_ws(p, ws, bytes);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // the loop state's flag (grid barriers) and the level tables' flags (staging copies)
  int flags[4] = {0, 0, 0, 0};
  JMG_CUDA(cudaMemcpyAsync(&flags[0], &ptr<LoopState>(ws, p->off_state)->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
  JMG_CUDA(cudaMemcpyAsync(&flags[1], &ptr<LvlTable<double>>(ws, p->off_tab64)->fault, sizeof(int),
                           cudaMemcpyDeviceToHost, s));
  if (p->mixed)
    JMG_CUDA(cudaMemcpyAsync(&flags[2], &ptr<LvlTable<float>>(ws, p->off_tab32)->fault, sizeof(int),
                             cudaMemcpyDeviceToHost, s));
  if (p->fcg && !p->mixed)
    JMG_CUDA(cudaMemcpyAsync(&flags[3], &ptr<LvlTable<double>>(ws, p->off_tab64z)->fault, sizeof(int),
                             cudaMemcpyDeviceToHost, s));
  JMG_CUDA(cudaStreamSynchronize(s));
  const int tma = p->dim == 3 && p->mixed ? sweep_tma3d_fault() : 0;
  if (flags[0] || flags[1] || flags[2] || flags[3] || tma)
    return set_err(JMG_ERR_TIMEOUT,
                   "a bounded device-side wait of the last solve on this workspace ran out (%s); its result is void",
                   flags[0] ? "a grid barrier of the middle-level kernel"
                            : tma ? "a plane copy of the one-pass 3D sweep" : "a staging copy of the coarse levels");
  return JMG_OK;
}

const char* jmg_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
