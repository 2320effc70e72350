// mg_adjoint_kernels.cu — reverse-mode kernels of the fixed-mode 2D cycle.
//
// The reference differentiates its fixed-mode solve with jax.vjp (solver_2d.py:18-26,
// tests/test_solver_2d.py:200-207). These kernels are the hand-written transposes of the
// forward operators in mg_common.cuh, on FP64 level arrays with the forward layout:
//   pb = adjoint of phi, rb = adjoint of rhs, T = scratch,
//   gacc / gwx / gwy = adjoints of A_cc and of the x / y face couplings.
// A Gauss-Seidel colour update phi[p] = (sum_q w_pq phi[q] - rhs[p]) / A_cc(p) has the
// transpose: t = pb[p] / A_cc(p); rb[p] -= t; gacc[p] -= t phi_new[p]; gw_pq += t phi_q;
// pb[q] += w_pq t for the neighbours q (other colour); pb[p] = 0. Each face joins one red
// and one black point, so within a colour every face gradient has a single writer.
#include "mg_adjoint_seg.h"
#include "mg_block.cuh"
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {


static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// points of one colour (2D: colour c means i + j == c mod 2), one thread per point
__device__ __forceinline__ bool colour_point(const Lvl<double>& a, int c, int& i, int& j) {
  i = blockIdx.y * blockDim.y + threadIdx.y + 2;
  j = 2 + ((i + c) & 1) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  return i <= a.my && j <= a.mx;
}

// ---- per-point bodies (the grid kernels and the single-block segments share them) ----

// transpose of one colour update, part 1, at (i, j): scale, rhs / coefficient adjoints,
// clear pb. nb: phi values the forward update read at the neighbours; nw: phi after it
__device__ __forceinline__ void adj_scale_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j,
                                             const double* __restrict__ nb, const double* __restrict__ nw) {
  const int P = a.P;
  const long long p = (long long)i * P + j;
  const double t = g.pb[p] * a.invd[p];
  g.T[p] = t;
  g.rb[p] -= t;
  g.gacc[p] -= t * nw[p];
  g.gwx[p - 1] += t * nb[p - 1];
  g.gwx[p] += t * nb[p + 1];
  g.gwy[p - P] += t * nb[p - P];
  g.gwy[p] += t * nb[p + P];
  g.pb[p] = 0.0;
}

// transpose of one colour update, part 2: the other colour gathers w_pq t_p (sign +1) or,
// for the defect, -w_pq d_p (sign -1)
__device__ __forceinline__ void adj_gather_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j, double sign) {
  const int P = a.P;
  const long long q = (long long)i * P + j;
  const double s = a.wx[q - 1] * g.T[q - 1] + a.wx[q] * g.T[q + 1] + a.wy[q - P] * g.T[q - P] + a.wy[q] * g.T[q + P];
  g.pb[q] += sign * s;
}

// transpose of defect + restriction, part 1, at the red point (i, j) (the only ones the
// restriction reads): d_bar = R^T rc_bar; rb += d_bar; pb += A_cc d_bar; coefficient adjoints
__device__ __forceinline__ void adj_restrict_red_pt(const Lvl<double>& a, const AdjLvl& g,
                                                    const double* __restrict__ phi, const Lvl<double>& c,
                                                    const double* __restrict__ rbc, int i, int j) {
  const int P = a.P, Pc = c.P;
  const long long p = (long long)i * P + j;
  double db = 0.0;
  if (i & 1) {  // (odd, odd): centre of coarse point ((i+1)/2, (j+1)/2), weight 1/4
    const int J = (i + 1) >> 1, I = (j + 1) >> 1;
    if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) db = 0.25 * rbc[(long long)J * Pc + I];
  } else {  // (even, even): diagonal neighbour of up to four coarse points, weight 1/16
    double s = 0.0;
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) {
        const int J = (i >> 1) + dj, I = (j >> 1) + di;
        if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) s += rbc[(long long)J * Pc + I];
      }
    db = 0.0625 * s;
  }
  g.T[p] = db;
  g.rb[p] += db;
  g.pb[p] += a.acc[p] * db;
  g.gacc[p] += db * phi[p];
  g.gwx[p - 1] -= db * phi[p - 1];
  g.gwx[p] -= db * phi[p + 1];
  g.gwy[p - P] -= db * phi[p - P];
  g.gwy[p] -= db * phi[p + P];
}

// transpose of phi_f += P(phi_c) at the coarse point (J, I) of the padded box: pb_c =
// P^T pb_f inside; also clears rb_c (a new coarse visit starts); zero on the frame
__device__ __forceinline__ void adj_prolong_pt(const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c,
                                               const AdjLvl& gc, int diag, int J, int I) {
  const long long q = (long long)J * c.P + I;
  double s = 0.0;
  if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) {
    const int P = f.P;
    const double* pb = gf.pb;
    const long long ctr = (long long)(2 * J - 1) * P + (2 * I - 1);
    s = pb[ctr];
    s += 0.5 * (pb[ctr + 1] + pb[ctr - 1]);
    s += 0.5 * (pb[ctr + P] + pb[ctr - P]);
    if (diag) s += 0.25 * (pb[ctr + P + 1] + pb[ctr - P + 1] + pb[ctr + P - 1] + pb[ctr - P - 1]);
  }
  gc.pb[q] = s;
  gc.rb[q] = 0.0;
}

// ---- grid-wide kernels ----------------------------------------------------------------

__global__ void k_adj_colour_scale(Lvl<double> a, AdjLvl g, int c, const double* __restrict__ nb,
                                   const double* __restrict__ nw) {
  int i, j;
  if (colour_point(a, c, i, j)) adj_scale_pt(a, g, i, j, nb, nw);
}

__global__ void k_adj_gather(Lvl<double> a, AdjLvl g, int c, double sign) {
  int i, j;
  if (colour_point(a, c, i, j)) adj_gather_pt(a, g, i, j, sign);
}

__global__ void k_adj_restrict_red(Lvl<double> a, AdjLvl g, const double* __restrict__ phi, Lvl<double> c,
                                   const double* __restrict__ rbc) {
  int i, j;
  if (colour_point(a, 0, i, j)) adj_restrict_red_pt(a, g, phi, c, rbc, i, j);
}

__global__ void k_adj_prolong(Lvl<double> f, AdjLvl gf, Lvl<double> c, AdjLvl gc, int diag) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I > c.mx + 2 || J > c.my + 2) return;
  adj_prolong_pt(f, gf, c, gc, diag, J, I);
}

// backward of the coefficient hierarchy of level l (solver_2d.py:326-421): A_cc adjoints
// go to the four faces and to lambda, faces to the two raw D values they average, raw D and
// lambda to the fine positions they were injected from. Dense outputs, accumulated.
__global__ void k_adj_hierarchy2d(Lvl<double> a, AdjLvl g, int level, double sx, double sy, int nx0, double* dbx,
                                  double* dby, double* dlam) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int mx = a.mx, my = a.my;
  if (I > mx + 2 || J > my + 2) return;
  const int P = a.P;
  auto inner = [&](int jj, int ii) { return jj >= 2 && jj <= my && ii >= 2 && ii <= mx; };
  auto gacc = [&](int jj, int ii) { return inner(jj, ii) ? g.gacc[(long long)jj * P + ii] : 0.0; };
  // total adjoint of the x face (jj, ii) between ii and ii+1, and of the y face (jj, ii)
  auto twx = [&](int jj, int ii) {
    if (jj < 1 || jj > my + 1 || ii < 0 || ii > mx + 1) return 0.0;
    return g.gwx[(long long)jj * P + ii] + gacc(jj, ii) + gacc(jj, ii + 1);
  };
  auto twy = [&](int jj, int ii) {
    if (jj < 0 || jj > my + 1 || ii < 1 || ii > mx + 1) return 0.0;
    return g.gwy[(long long)jj * P + ii] + gacc(jj, ii) + gacc(jj + 1, ii);
  };
  // raw D of this level at (J, I) feeds x faces (J, I) and (J, I-1), y faces (J, I) and (J-1, I)
  const double rx = 0.5 * sx * (twx(J, I) + twx(J, I - 1));
  const double ry = 0.5 * sy * (twy(J, I) + twy(J - 1, I));
  const double rl = gacc(J, I);
  long long f;
  if (level == 0) {
    f = (long long)J * nx0 + I;
  } else {
    if (J < 1 || J > my + 1 || I < 1 || I > mx + 1) return;  // injected ring only
    f = (long long)(((J - 1) << level) + 1) * nx0 + (((I - 1) << level) + 1);
  }
  dbx[f] += rx;
  dby[f] += ry;
  dlam[f] += rl;
}

void adj_sweep(const Lvl<double>& a, const AdjLvl& g, const double* before, const double* after, cudaStream_t s) {
  dim3 b(64, 4), gr(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4));
  // reverse of the forward order: black (colour 1) then red (colour 0)
  k_adj_colour_scale<<<gr, b, 0, s>>>(a, g, 1, after, after);   // black read the new red values
  k_adj_gather<<<gr, b, 0, s>>>(a, g, 0, 1.0);
  k_adj_colour_scale<<<gr, b, 0, s>>>(a, g, 0, before, after);  // red read the old black values
  k_adj_gather<<<gr, b, 0, s>>>(a, g, 1, 1.0);
}

void adj_restrict(const Lvl<double>& a, const AdjLvl& g, const double* phi, const Lvl<double>& c, const AdjLvl& gc,
                  cudaStream_t s) {
  dim3 b(64, 4), gr(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4));
  k_adj_restrict_red<<<gr, b, 0, s>>>(a, g, phi, c, gc.rb);
  k_adj_gather<<<gr, b, 0, s>>>(a, g, 1, -1.0);
}

void adj_prolong(const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c, const AdjLvl& gc, int diag,
                 cudaStream_t s) {
  dim3 b(32, 8), gr(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8));
  k_adj_prolong<<<gr, b, 0, s>>>(f, gf, c, gc, diag);
}

void adj_hierarchy2d(const Lvl<double>& a, const AdjLvl& g, int level, double sx, double sy, int nx0, double* dbx,
                     double* dby, double* dlam, cudaStream_t s) {
  dim3 b(32, 8), gr(cdiv(a.mx + 3, 32), cdiv(a.my + 3, 8));
  k_adj_hierarchy2d<<<gr, b, 0, s>>>(a, g, level, sx, sy, nx0, dbx, dby, dlam);
}

// ---- single-block segments ------------------------------------------------------------
// A run of tape operators on the small levels (one block's worth of points) executes in
// one launch: the forward with its snapshots, or the reverse, one pass per barrier. The
// passes evaluate the per-point bodies above (adjoint) and mg_block.cuh (forward), the
// same as the grid-wide kernels, so the results are the same bits.

template <typename F>
__device__ __forceinline__ void blk_colour(const Lvl<double>& a, int c, F&& body) {
  const int hx = a.mx / 2, n = hx * (a.my - 1);
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = 2 + t / hx;
    const int j = 2 + ((i + c) & 1) + 2 * (t % hx);
    if (j <= a.mx) body(i, j);
  }
  __syncthreads();
}

__device__ void blk_adj_sweep(const Lvl<double>& a, const AdjLvl& g, const double* before, const double* after) {
  // reverse of the forward order: black (colour 1) then red (colour 0)
  blk_colour(a, 1, [&](int i, int j) { adj_scale_pt(a, g, i, j, after, after); });
  blk_colour(a, 0, [&](int i, int j) { adj_gather_pt(a, g, i, j, 1.0); });
  blk_colour(a, 0, [&](int i, int j) { adj_scale_pt(a, g, i, j, before, after); });
  blk_colour(a, 1, [&](int i, int j) { adj_gather_pt(a, g, i, j, 1.0); });
}

__device__ void blk_adj_restrict(const Lvl<double>& a, const AdjLvl& g, const double* phi, const Lvl<double>& c,
                                 const AdjLvl& gc) {
  blk_colour(a, 0, [&](int i, int j) { adj_restrict_red_pt(a, g, phi, c, gc.rb, i, j); });
  blk_colour(a, 1, [&](int i, int j) { adj_gather_pt(a, g, i, j, -1.0); });
}

__device__ void blk_adj_prolong(const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c, const AdjLvl& gc,
                                int diag) {
  const int nx = c.mx + 3, n = nx * (c.my + 3);
  for (int t = threadIdx.x; t < n; t += blockDim.x) adj_prolong_pt(f, gf, c, gc, diag, t / nx, t % nx);
  __syncthreads();
}

// the tables and the segment, staged in shared memory (they are read at every operator)
struct AdjSegStage {
  AdjTables tab;
  AdjSeg seg;
};

__device__ void stage_seg(AdjSegStage* st, const AdjTables* tabs, const AdjSeg* seg) {
  const int n1 = (int)(sizeof(AdjTables) / sizeof(int)), n2 = (int)(sizeof(AdjSeg) / sizeof(int));
  const int* a = reinterpret_cast<const int*>(tabs);
  const int* b = reinterpret_cast<const int*>(seg);
  int* da = reinterpret_cast<int*>(&st->tab);
  int* db = reinterpret_cast<int*>(&st->seg);
  for (int k = threadIdx.x; k < n1; k += blockDim.x) da[k] = a[k];
  for (int k = threadIdx.x; k < n2; k += blockDim.x) db[k] = b[k];
  __syncthreads();
}

__global__ void __launch_bounds__(1024) k_adj_seg_fwd(const AdjTables* tabs, const AdjSeg* seg, int snapshots,
                                                     int diag) {
  __shared__ AdjSegStage st;
  stage_seg(&st, tabs, seg);
  for (int o = 0; o < st.seg.n; ++o) {
    const AdjSegOp op = st.seg.op[o];
    const Lvl<double>& a = st.tab.lv.l[op.lev];
    if (op.kind == kAdjOpRestrict) {
      blk_restrict<double, 2>(a, st.tab.lv.l[op.lev + 1]);
      continue;
    }
    if (op.kind == kAdjOpSweep) blk_sweep<double, 2>(a);
    else blk_prolong<double, 2>(a, st.tab.lv.l[op.lev + 1], diag != 0);
    if (snapshots) {
      const int n = a.P * (a.my + 3);
      for (int t = threadIdx.x; t < n; t += blockDim.x) op.after[t] = a.phi[t];
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(1024) k_adj_seg_rev(const AdjTables* tabs, const AdjSeg* seg, int diag) {
  __shared__ AdjSegStage st;
  stage_seg(&st, tabs, seg);
  for (int o = st.seg.n - 1; o >= 0; --o) {
    const AdjSegOp op = st.seg.op[o];
    const Lvl<double>& a = st.tab.lv.l[op.lev];
    const AdjLvl& g = st.tab.g[op.lev];
    if (op.kind == kAdjOpSweep) blk_adj_sweep(a, g, op.before, op.after);
    else if (op.kind == kAdjOpProlong) blk_adj_prolong(a, g, st.tab.lv.l[op.lev + 1], st.tab.g[op.lev + 1], diag);
    else blk_adj_restrict(a, g, op.before, st.tab.lv.l[op.lev + 1], st.tab.g[op.lev + 1]);
  }
}

template <typename V>
__global__ void k_adj_store(V v, V* dst) {
  const int n = (int)(sizeof(V) / sizeof(int));
  const int* src = reinterpret_cast<const int*>(&v);
  int* d = reinterpret_cast<int*>(dst);
  for (int k = threadIdx.x; k < n; k += blockDim.x) d[k] = src[k];
}

void adj_store_tables(const AdjTables& t, AdjTables* dst, cudaStream_t s) { k_adj_store<<<1, 256, 0, s>>>(t, dst); }
void adj_store_seg(const AdjSeg& g, AdjSeg* dst, cudaStream_t s) { k_adj_store<<<1, 256, 0, s>>>(g, dst); }
void adj_seg_fwd(const AdjTables* t, const AdjSeg* g, bool snapshots, int diag, cudaStream_t s) {
  k_adj_seg_fwd<<<1, 1024, 0, s>>>(t, g, snapshots ? 1 : 0, diag);
}
void adj_seg_rev(const AdjTables* t, const AdjSeg* g, int diag, cudaStream_t s) {
  k_adj_seg_rev<<<1, 1024, 0, s>>>(t, g, diag);
}

}  // namespace jmg
