// mg_adjoint_kernels.cu — reverse-mode kernels of the fixed-mode cycle: 2D with the
// 5-point and the 9-point (D_xy) stencil, 3D with the 7-point stencil.
//
// The reference differentiates its fixed-mode solve with jax.vjp (solver_2d.py:18-26,
// tests/test_solver_2d.py:200-207; solver_3d.py:468-470). These kernels are the
// hand-written transposes of the forward operators in mg_common.cuh, on FP64 level arrays
// with the forward layout:
//   pb = adjoint of phi, rb = adjoint of rhs, T = scratch, gacc = adjoint of A_cc,
//   gwx / gwy / gwz = adjoints of the face couplings, gxll .. gxrr = adjoints of the
//   diagonal couplings of the 9-point stencil.
// A Gauss-Seidel update phi[p] = (sum_q w_pq phi[q] - rhs[p]) / A_cc(p) has the transpose:
// t = pb[p] / A_cc(p); rb[p] -= t; gacc[p] -= t phi_new[p]; gw_pq += t phi_q; pb[q] += w_pq t
// for the neighbours q; pb[p] = 0. A pass updates points that never neighbour each other
// (a colour of the 5- and 7-point stencils, a sub-lattice of the 9-point one), so every
// coupling gradient has a single writer within a pass; the neighbours' part ("gather") is
// a second pass over the points that read T, which only ever reads T at the updated points.
#include "mg_adjoint_seg.h"
#include "mg_block.cuh"
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

static_assert(sizeof(AdjTables) <= 4096, "the tables are passed as one kernel parameter");

static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// ---- 2D per-point bodies (the grid kernels and the single-block segments share them) --

// points of one colour (2D: colour c means i + j == c mod 2), one thread per point
__device__ __forceinline__ bool colour_point(const Lvl<double>& a, int c, int& i, int& j) {
  i = blockIdx.y * blockDim.y + threadIdx.y + 2;
  j = 2 + ((i + c) & 1) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  return i <= a.my && j <= a.mx;
}

// The 9-point sweep updates the sub-lattices in the reference's order (solver_2d.py:684),
// by (row, column) parity: (1,1), (0,0), (0,1), (1,0); sub-lattice k's row / column parity:
__host__ __device__ constexpr int sl_row(int k) { return k == 0 || k == 3 ? 1 : 0; }
__host__ __device__ constexpr int sl_col(int k) { return k == 0 || k == 2 ? 1 : 0; }

// transpose of one update, part 1, at (i, j): scale, rhs / coefficient adjoints, clear pb.
// nf / nd: phi values the forward update read at the face / diagonal neighbours (the
// states before or after the sweep, by the neighbour's place in the pass order); nw: phi
// after the sweep (the updated value at (i, j))
__device__ __forceinline__ void adj_scale_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j,
                                             const double* __restrict__ nf, const double* __restrict__ nd,
                                             const double* __restrict__ nw) {
  const int P = a.P;
  const long long p = (long long)i * P + j;
  const double t = g.pb[p] * a.invd[p];
  g.T[p] = t;
  g.rb[p] -= t;
  g.gacc[p] -= t * nw[p];
  g.gwx[p - 1] += t * nf[p - 1];
  g.gwx[p] += t * nf[p + 1];
  g.gwy[p - P] += t * nf[p - P];
  g.gwy[p] += t * nf[p + P];
  if (a.xll) {
    g.gxll[p] += t * nd[p - P - 1];
    g.gxrl[p] += t * nd[p - P + 1];
    g.gxlr[p] += t * nd[p + P - 1];
    g.gxrr[p] += t * nd[p + P + 1];
  }
  g.pb[p] = 0.0;
}

// transpose of one update, part 2: the point q gathers w_pq t_p (sign +1) or, for the
// defect, -w_pq d_p (sign -1) from the updated points p among its face neighbours
__device__ __forceinline__ void adj_gather_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j, double sign) {
  const int P = a.P;
  const long long q = (long long)i * P + j;
  const double s = a.wx[q - 1] * g.T[q - 1] + a.wx[q] * g.T[q + 1] + a.wy[q - P] * g.T[q - P] + a.wy[q] * g.T[q + P];
  g.pb[q] += sign * s;
}

// the same from chosen neighbour groups of the 9-point stencil: north / south (ns), east
// / west (ew), the diagonals (dg). q is the SW neighbour of p = q+P+1 (A_ll(p)), SE of
// q+P-1 (A_rl), NW of q-P+1 (A_lr) and NE of q-P-1 (A_rr).
__device__ __forceinline__ void adj_gather9_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j, bool ns,
                                               bool ew, bool dg, double sign) {
  const int P = a.P;
  const long long q = (long long)i * P + j;
  const double* T = g.T;
  double s = 0.0;
  if (ns) s += a.wy[q - P] * T[q - P] + a.wy[q] * T[q + P];
  if (ew) s += a.wx[q - 1] * T[q - 1] + a.wx[q] * T[q + 1];
  if (dg)
    s += a.xll[q + P + 1] * T[q + P + 1] + a.xrl[q + P - 1] * T[q + P - 1] + a.xlr[q - P + 1] * T[q - P + 1] +
         a.xrr[q - P - 1] * T[q - P - 1];
  g.pb[q] += sign * s;
}

// gather of sweep pass k (9-point): q reads T from its neighbours in sub-lattice k, which
// sit north / south of it when only the row parity differs, east / west when only the
// column parity differs, diagonally when both differ
__device__ __forceinline__ void adj_gather_sub_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j, int k) {
  const bool dr = (i & 1) != sl_row(k), dc = (j & 1) != sl_col(k);
  if (dr || dc) adj_gather9_pt(a, g, i, j, dr && !dc, dc && !dr, dr && dc, 1.0);
}

// gather after the restriction's transpose: the defect was read at the red points (i + j
// even); black points take it from their four faces, red points (9-point) from their
// diagonals
__device__ __forceinline__ void adj_gather_defect_pt(const Lvl<double>& a, const AdjLvl& g, int i, int j) {
  if ((i + j) & 1) adj_gather9_pt(a, g, i, j, true, true, false, -1.0);
  else if (a.xll) adj_gather9_pt(a, g, i, j, false, false, true, -1.0);
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
  if (a.xll) {  // the defect subtracts the off-diagonal part (solver_2d.py:637-642)
    g.gxll[p] -= db * phi[p - P - 1];
    g.gxrl[p] -= db * phi[p - P + 1];
    g.gxlr[p] -= db * phi[p + P - 1];
    g.gxrr[p] -= db * phi[p + P + 1];
  }
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

// ---- 3D per-point bodies ----------------------------------------------------------------

// points of one colour (3D: colour 0 is i+j+k odd, the reference's first four
// sub-lattices), one thread per point; grid z walks planes
__device__ __forceinline__ bool colour_point3(const Lvl<double>& a, int c, int& k, int& j, int& i) {
  k = blockIdx.z + 2;
  j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int par = (first_color_parity<3>() + c) & 1;
  i = 2 + ((j + k + par) & 1) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  return j <= a.my && k <= a.mz && i <= a.mx;
}

__device__ __forceinline__ void adj_scale_pt3(const Lvl<double>& a, const AdjLvl& g, long long p,
                                              const double* __restrict__ nb, const double* __restrict__ nw) {
  const int P = a.P;
  const long long S = a.S;
  const double t = g.pb[p] * a.invd[p];
  g.T[p] = t;
  g.rb[p] -= t;
  g.gacc[p] -= t * nw[p];
  g.gwx[p - 1] += t * nb[p - 1];
  g.gwx[p] += t * nb[p + 1];
  g.gwy[p - P] += t * nb[p - P];
  g.gwy[p] += t * nb[p + P];
  g.gwz[p - S] += t * nb[p - S];
  g.gwz[p] += t * nb[p + S];
  g.pb[p] = 0.0;
}

__device__ __forceinline__ void adj_gather_pt3(const Lvl<double>& a, const AdjLvl& g, long long q, double sign) {
  const int P = a.P;
  const long long S = a.S;
  const double* T = g.T;
  double s = a.wx[q - 1] * T[q - 1] + a.wx[q] * T[q + 1];
  s += a.wy[q - P] * T[q - P] + a.wy[q] * T[q + P];
  s += a.wz[q - S] * T[q - S] + a.wz[q] * T[q + S];
  g.pb[q] += sign * s;
}

// transpose of defect + restriction at the red point (k, j, i) (solver_3d.py:622-652):
// with three odd indices it is the centre of one coarse point (weight 1/8), with one odd
// index an edge-diagonal neighbour of the up to four coarse points around it (1/32 each)
__device__ __forceinline__ void adj_restrict_red_pt3(const Lvl<double>& a, const AdjLvl& g,
                                                     const double* __restrict__ phi, const Lvl<double>& c,
                                                     const double* __restrict__ rbc, int k, int j, int i) {
  const int P = a.P, Pc = c.P;
  const long long S = a.S, Sc = c.S;
  const long long p = (long long)k * S + (long long)j * P + i;
  auto in = [&](int K, int J, int I) { return K >= 2 && K <= c.mz && J >= 2 && J <= c.my && I >= 2 && I <= c.mx; };
  auto rc = [&](int K, int J, int I) { return in(K, J, I) ? rbc[(long long)K * Sc + (long long)J * Pc + I] : 0.0; };
  double db;
  if ((k & 1) && (j & 1) && (i & 1)) {
    db = 0.125 * rc((k + 1) >> 1, (j + 1) >> 1, (i + 1) >> 1);
  } else {
    // the odd axis fixes its coarse index, the two even ones take f/2 and f/2 + 1
    double s = 0.0;
    for (int u = 0; u < 2; ++u)
      for (int v = 0; v < 2; ++v) {
        if (k & 1) s += rc((k + 1) >> 1, (j >> 1) + u, (i >> 1) + v);
        else if (j & 1) s += rc((k >> 1) + u, (j + 1) >> 1, (i >> 1) + v);
        else s += rc((k >> 1) + u, (j >> 1) + v, (i + 1) >> 1);
      }
    db = 0.03125 * s;
  }
  g.T[p] = db;
  g.rb[p] += db;
  g.pb[p] += a.acc[p] * db;
  g.gacc[p] += db * phi[p];
  g.gwx[p - 1] -= db * phi[p - 1];
  g.gwx[p] -= db * phi[p + 1];
  g.gwy[p - P] -= db * phi[p - P];
  g.gwy[p] -= db * phi[p + P];
  g.gwz[p - S] -= db * phi[p - S];
  g.gwz[p] -= db * phi[p + S];
}

// transpose of phi_f += P(phi_c) at the coarse point (K, J, I) of the padded box
// (solver_3d.py:654-677): the fine points 2K-1+dk, 2J-1+dj, 2I-1+di (d in -1..1) read it
// with weight 1/2 per nonzero offset; the points with two nonzero offsets only when the
// bilinear class is computed (nu2 <= 0). Clears rb_c; zero on the frame.
__device__ __forceinline__ void adj_prolong_pt3(const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c,
                                                const AdjLvl& gc, int bilinear, int K, int J, int I) {
  const long long q = (long long)K * c.S + (long long)J * c.P + I;
  double s = 0.0;
  if (K >= 2 && K <= c.mz && J >= 2 && J <= c.my && I >= 2 && I <= c.mx) {
    const int P = f.P;
    const long long S = f.S;
    const long long ctr = (long long)(2 * K - 1) * S + (long long)(2 * J - 1) * P + (2 * I - 1);
    const double* pb = gf.pb;
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          const int ne = (dk != 0) + (dj != 0) + (di != 0);
          if (ne == 2 && !bilinear) continue;
          const double w = ne == 0 ? 1.0 : ne == 1 ? 0.5 : ne == 2 ? 0.25 : 0.125;
          s += w * pb[ctr + dk * S + dj * P + di];
        }
  }
  gc.pb[q] = s;
  gc.rb[q] = 0.0;
}

// ---- grid-wide kernels ----------------------------------------------------------------

__global__ void k_adj_colour_scale(Lvl<double> a, AdjLvl g, int c, const double* __restrict__ nb,
                                   const double* __restrict__ nw) {
  int i, j;
  if (colour_point(a, c, i, j)) adj_scale_pt(a, g, i, j, nb, nb, nw);
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

// 9-point: scale of sub-lattice k (rows of parity sl_row(k), columns of parity sl_col(k))
__global__ void k_adj_sub_scale(Lvl<double> a, AdjLvl g, int k, const double* __restrict__ nf,
                                const double* __restrict__ nd, const double* __restrict__ nw) {
  const int i = 2 + sl_row(k) + 2 * (blockIdx.y * blockDim.y + threadIdx.y);
  const int j = 2 + sl_col(k) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (i <= a.my && j <= a.mx) adj_scale_pt(a, g, i, j, nf, nd, nw);
}

// 9-point gathers over every interior point: of sweep pass k (k >= 0) or, with k < 0, of
// the restriction's defect
__global__ void k_adj_gather9(Lvl<double> a, AdjLvl g, int k) {
  const int j = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = 2 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > a.my || j > a.mx) return;
  if (k >= 0) adj_gather_sub_pt(a, g, i, j, k);
  else adj_gather_defect_pt(a, g, i, j);
}

__global__ void k_adj_colour_scale3(Lvl<double> a, AdjLvl g, int c, const double* __restrict__ nb,
                                    const double* __restrict__ nw) {
  int k, j, i;
  if (colour_point3(a, c, k, j, i)) adj_scale_pt3(a, g, (long long)k * a.S + (long long)j * a.P + i, nb, nw);
}

__global__ void k_adj_gather3(Lvl<double> a, AdjLvl g, int c, double sign) {
  int k, j, i;
  if (colour_point3(a, c, k, j, i)) adj_gather_pt3(a, g, (long long)k * a.S + (long long)j * a.P + i, sign);
}

__global__ void k_adj_restrict_red3(Lvl<double> a, AdjLvl g, const double* __restrict__ phi, Lvl<double> c,
                                    const double* __restrict__ rbc) {
  int k, j, i;
  if (colour_point3(a, 0, k, j, i)) adj_restrict_red_pt3(a, g, phi, c, rbc, k, j, i);
}

__global__ void k_adj_prolong3(Lvl<double> f, AdjLvl gf, Lvl<double> c, AdjLvl gc, int bilinear) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I > c.mx + 2 || J > c.my + 2) return;
  adj_prolong_pt3(f, gf, c, gc, bilinear, K, J, I);
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

// backward of the diagonal couplings of level l (2D with D_xy, solver_2d.py:410-416):
//   A_ll(J,I) = (Dxy(J,I-1) + Dxy(J-1,I)) c    A_lr(J,I) = -(Dxy(J,I-1) + Dxy(J+1,I)) c
//   A_rl(J,I) = -(Dxy(J,I+1) + Dxy(J-1,I)) c   A_rr(J,I) = (Dxy(J,I+1) + Dxy(J+1,I)) c
// on J, I in 1..m+1 from the raw injected D_xy; the adjoint of the raw value at (J, I)
// collects the four couplings of each of its four face neighbours that read it.
__global__ void k_adj_hier_xy2d(Lvl<double> a, AdjLvl g, int level, double cxy, int nx0, double* dxy) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int mx = a.mx, my = a.my;
  if (I > mx + 2 || J > my + 2) return;
  const int P = a.P;
  auto at = [&](const double* arr, int jj, int ii) {
    return (jj >= 1 && jj <= my + 1 && ii >= 1 && ii <= mx + 1) ? arr[(long long)jj * P + ii] : 0.0;
  };
  double r = at(g.gxll, J, I + 1) - at(g.gxlr, J, I + 1);  // west neighbour of (J, I+1)
  r += at(g.gxrr, J, I - 1) - at(g.gxrl, J, I - 1);         // east neighbour of (J, I-1)
  r += at(g.gxll, J + 1, I) - at(g.gxrl, J + 1, I);         // south neighbour of (J+1, I)
  r += at(g.gxrr, J - 1, I) - at(g.gxlr, J - 1, I);         // north neighbour of (J-1, I)
  r *= cxy;
  long long f;
  if (level == 0) {
    f = (long long)J * nx0 + I;
  } else {
    if (J < 1 || J > my + 1 || I < 1 || I > mx + 1) return;
    f = (long long)(((J - 1) << level) + 1) * nx0 + (((I - 1) << level) + 1);
  }
  dxy[f] += r;
}

// backward of the 3D coefficient hierarchy of level l (solver_3d.py:338-429). Level 0's
// face couplings are the raw cell D times idel^2; level l >= 1 face-averages the values it
// injects from level l-1 (the raw D for l = 1, level l-1's averaged D otherwise), so the
// adjoints run down the chain: the levels are processed coarsest first, and level l adds
// the adjoint of each injected value to level l-1's averaged-D adjoint (gprev) or, for
// l = 1, to the dense D adjoint. gcur holds what level l+1 added to this level's (nullptr
// at the coarsest). lambda is injected from level 0 at every level.
struct AdjHier3 {
  Lvl<double> a;
  AdjLvl g;
  int level;
  double sq[3];
  int nx0, ny0;           // dense level-0 extents
  int Pp;                 // level l-1's pitch and plane stride (targets of gprev)
  long long Sp;
  double* gprev[3];
  const double* gcur[3];
  double* dbar[3];
  double* dlam;
};

__global__ void k_adj_hierarchy3d(AdjHier3 h) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  const Lvl<double>& a = h.a;
  const int mx = a.mx, my = a.my, mz = a.mz;
  if (I > mx + 2 || J > my + 2) return;
  const int P = a.P;
  const long long S = a.S;
  auto idx = [&](int kk, int jj, int ii) { return (long long)kk * S + (long long)jj * P + ii; };
  auto box = [&](int kk, int jj, int ii) {
    return kk >= 0 && kk <= mz + 2 && jj >= 0 && jj <= my + 2 && ii >= 0 && ii <= mx + 2;
  };
  auto gacc = [&](int kk, int jj, int ii) {
    return (kk >= 2 && kk <= mz && jj >= 2 && jj <= my && ii >= 2 && ii <= mx) ? h.g.gacc[idx(kk, jj, ii)] : 0.0;
  };
  const double* gw[3] = {h.g.gwx, h.g.gwy, h.g.gwz};
  // adjoint of this level's D of component c at (kk, jj, ii): through the face coupling
  // (gw, and A_cc on both sides of the face) and through level l+1's injection
  auto gd = [&](int c, int kk, int jj, int ii) {
    if (!box(kk, jj, ii)) return 0.0;
    const int dk = c == 2, dj = c == 1, di = c == 0;
    const double tw = gw[c][idx(kk, jj, ii)] + gacc(kk, jj, ii) + gacc(kk + dk, jj + dj, ii + di);
    return h.sq[c] * tw + (h.gcur[c] ? h.gcur[c][idx(kk, jj, ii)] : 0.0);
  };
  const long long nxy0 = (long long)h.nx0 * h.ny0;
  if (K >= 2 && K <= mz && J >= 2 && J <= my && I >= 2 && I <= mx) {
    const long long f = h.level == 0 ? K * nxy0 + (long long)J * h.nx0 + I
                                     : (long long)(((K - 1) << h.level) + 1) * nxy0 +
                                           (long long)(((J - 1) << h.level) + 1) * h.nx0 + (((I - 1) << h.level) + 1);
    h.dlam[f] += h.g.gacc[idx(K, J, I)];
  }
  if (h.level == 0) {
    const long long f = K * nxy0 + (long long)J * h.nx0 + I;
    for (int c = 0; c < 3; ++c) h.dbar[c][f] += gd(c, K, J, I);
    return;
  }
  if (K < 1 || K > mz + 1 || J < 1 || J > my + 1 || I < 1 || I > mx + 1) return;  // injected cube only
  // the injected value at (K, J, I) enters the averages at (K, J, I) and one step down the axis
  double gi[3];
  gi[0] = 0.5 * (gd(0, K, J, I) + gd(0, K, J, I - 1));
  gi[1] = 0.5 * (gd(1, K, J, I) + gd(1, K, J - 1, I));
  gi[2] = 0.5 * (gd(2, K, J, I) + gd(2, K - 1, J, I));
  if (h.level == 1) {
    const long long f = (long long)(2 * K - 1) * nxy0 + (long long)(2 * J - 1) * h.nx0 + (2 * I - 1);
    for (int c = 0; c < 3; ++c) h.dbar[c][f] += gi[c];
  } else {
    const long long f = (long long)(2 * K - 1) * h.Sp + (long long)(2 * J - 1) * h.Pp + (2 * I - 1);
    for (int c = 0; c < 3; ++c) h.gprev[c][f] += gi[c];
  }
}

// ---- launchers ------------------------------------------------------------------------

void adj_sweep(int dim, const Lvl<double>& a, const AdjLvl& g, const double* before, const double* after,
               cudaStream_t s) {
  if (dim == 3) {
    dim3 b(64, 4, 1), gr(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4), a.mz - 1);
    k_adj_colour_scale3<<<gr, b, 0, s>>>(a, g, 1, after, after);
    k_adj_gather3<<<gr, b, 0, s>>>(a, g, 0, 1.0);
    k_adj_colour_scale3<<<gr, b, 0, s>>>(a, g, 0, before, after);
    k_adj_gather3<<<gr, b, 0, s>>>(a, g, 1, 1.0);
    return;
  }
  if (a.xll) {
    // the four sub-lattice passes in reverse; pass k read the faces after the sweep for
    // k >= 2 and the diagonals after it for k = 1, 3
    dim3 b(64, 4), gs(cdiv(a.mx / 2 + 1, 64), cdiv(a.my / 2 + 1, 4)), ga(cdiv(a.mx - 1, 64), cdiv(a.my - 1, 4));
    for (int k = 3; k >= 0; --k) {
      k_adj_sub_scale<<<gs, b, 0, s>>>(a, g, k, k >= 2 ? after : before, (k & 1) ? after : before, after);
      k_adj_gather9<<<ga, b, 0, s>>>(a, g, k);
    }
    return;
  }
  dim3 b(64, 4), gr(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4));
  // reverse of the forward order: black (colour 1) then red (colour 0)
  k_adj_colour_scale<<<gr, b, 0, s>>>(a, g, 1, after, after);   // black read the new red values
  k_adj_gather<<<gr, b, 0, s>>>(a, g, 0, 1.0);
  k_adj_colour_scale<<<gr, b, 0, s>>>(a, g, 0, before, after);  // red read the old black values
  k_adj_gather<<<gr, b, 0, s>>>(a, g, 1, 1.0);
}

void adj_restrict(int dim, const Lvl<double>& a, const AdjLvl& g, const double* phi, const Lvl<double>& c,
                  const AdjLvl& gc, cudaStream_t s) {
  if (dim == 3) {
    dim3 b(64, 4, 1), gr(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4), a.mz - 1);
    k_adj_restrict_red3<<<gr, b, 0, s>>>(a, g, phi, c, gc.rb);
    k_adj_gather3<<<gr, b, 0, s>>>(a, g, 1, -1.0);
    return;
  }
  dim3 b(64, 4), gr(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4));
  k_adj_restrict_red<<<gr, b, 0, s>>>(a, g, phi, c, gc.rb);
  if (a.xll) {
    dim3 ga(cdiv(a.mx - 1, 64), cdiv(a.my - 1, 4));
    k_adj_gather9<<<ga, b, 0, s>>>(a, g, -1);
  } else {
    k_adj_gather<<<gr, b, 0, s>>>(a, g, 1, -1.0);
  }
}

void adj_prolong(int dim, const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c, const AdjLvl& gc, int diag,
                 cudaStream_t s) {
  if (dim == 3) {
    dim3 b(32, 8, 1), gr(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8), c.mz + 3);
    k_adj_prolong3<<<gr, b, 0, s>>>(f, gf, c, gc, diag);
    return;
  }
  dim3 b(32, 8), gr(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8));
  k_adj_prolong<<<gr, b, 0, s>>>(f, gf, c, gc, diag);
}

void adj_hierarchy2d(const Lvl<double>& a, const AdjLvl& g, int level, double sx, double sy, int nx0, double* dbx,
                     double* dby, double* dlam, cudaStream_t s) {
  dim3 b(32, 8), gr(cdiv(a.mx + 3, 32), cdiv(a.my + 3, 8));
  k_adj_hierarchy2d<<<gr, b, 0, s>>>(a, g, level, sx, sy, nx0, dbx, dby, dlam);
}

void adj_hier_xy2d(const Lvl<double>& a, const AdjLvl& g, int level, double cxy, int nx0, double* dxy,
                   cudaStream_t s) {
  dim3 b(32, 8), gr(cdiv(a.mx + 3, 32), cdiv(a.my + 3, 8));
  k_adj_hier_xy2d<<<gr, b, 0, s>>>(a, g, level, cxy, nx0, dxy);
}

void adj_hierarchy3d(const Lvl<double>& a, const AdjLvl& g, int level, const double* sq, int nx0, int ny0,
                     const Lvl<double>* prev, double* const* gprev, const double* const* gcur, double* const* dbar,
                     double* dlam, cudaStream_t s) {
  AdjHier3 h;
  h.a = a;
  h.g = g;
  h.level = level;
  h.nx0 = nx0;
  h.ny0 = ny0;
  h.Pp = prev ? prev->P : 0;
  h.Sp = prev ? prev->S : 0;
  for (int c = 0; c < 3; ++c) {
    h.sq[c] = sq[c];
    h.gprev[c] = gprev ? gprev[c] : nullptr;
    h.gcur[c] = gcur ? gcur[c] : nullptr;
    h.dbar[c] = dbar[c];
  }
  h.dlam = dlam;
  dim3 b(32, 8, 1), gr(cdiv(a.mx + 3, 32), cdiv(a.my + 3, 8), a.mz + 3);
  k_adj_hierarchy3d<<<gr, b, 0, s>>>(h);
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

// every interior point (9-point gathers)
template <typename F>
__device__ __forceinline__ void blk_all(const Lvl<double>& a, F&& body) {
  const int nx = a.mx - 1, n = nx * (a.my - 1);
  for (int t = threadIdx.x; t < n; t += blockDim.x) body(2 + t / nx, 2 + t % nx);
  __syncthreads();
}

// 3D: the points of colour c (0: i+j+k odd), as linear indices
template <typename F>
__device__ __forceinline__ void blk_colour3(const Lvl<double>& a, int c, F&& body) {
  const int hx = a.mx / 2, ny = a.my - 1, nz = a.mz - 1, n = hx * ny * nz;
  const int par = (first_color_parity<3>() + c) & 1;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int r = t / hx;
    const int j = 2 + r % ny, k = 2 + r / ny;
    const int i = 2 + ((j + k + par) & 1) + 2 * (t % hx);
    if (i <= a.mx) body(k, j, i, (long long)k * a.S + (long long)j * a.P + i);
  }
  __syncthreads();
}

template <int DIM>
__device__ void blk_adj_sweep(const Lvl<double>& a, const AdjLvl& g, const double* before, const double* after) {
  if (DIM == 3) {
    blk_colour3(a, 1, [&](int, int, int, long long p) { adj_scale_pt3(a, g, p, after, after); });
    blk_colour3(a, 0, [&](int, int, int, long long p) { adj_gather_pt3(a, g, p, 1.0); });
    blk_colour3(a, 0, [&](int, int, int, long long p) { adj_scale_pt3(a, g, p, before, after); });
    blk_colour3(a, 1, [&](int, int, int, long long p) { adj_gather_pt3(a, g, p, 1.0); });
  } else if (a.xll) {
    for (int k = 3; k >= 0; --k) {
      const double* nf = k >= 2 ? after : before;
      const double* nd = (k & 1) ? after : before;
      blk_all(a, [&](int i, int j) {
        if ((i & 1) == sl_row(k) && (j & 1) == sl_col(k)) adj_scale_pt(a, g, i, j, nf, nd, after);
      });
      blk_all(a, [&](int i, int j) { adj_gather_sub_pt(a, g, i, j, k); });
    }
  } else {
    // reverse of the forward order: black (colour 1) then red (colour 0)
    blk_colour(a, 1, [&](int i, int j) { adj_scale_pt(a, g, i, j, after, after, after); });
    blk_colour(a, 0, [&](int i, int j) { adj_gather_pt(a, g, i, j, 1.0); });
    blk_colour(a, 0, [&](int i, int j) { adj_scale_pt(a, g, i, j, before, before, after); });
    blk_colour(a, 1, [&](int i, int j) { adj_gather_pt(a, g, i, j, 1.0); });
  }
}

template <int DIM>
__device__ void blk_adj_restrict(const Lvl<double>& a, const AdjLvl& g, const double* phi, const Lvl<double>& c,
                                 const AdjLvl& gc) {
  if (DIM == 3) {
    blk_colour3(a, 0, [&](int k, int j, int i, long long) { adj_restrict_red_pt3(a, g, phi, c, gc.rb, k, j, i); });
    blk_colour3(a, 1, [&](int, int, int, long long p) { adj_gather_pt3(a, g, p, -1.0); });
  } else {
    blk_colour(a, 0, [&](int i, int j) { adj_restrict_red_pt(a, g, phi, c, gc.rb, i, j); });
    if (a.xll) blk_all(a, [&](int i, int j) { adj_gather_defect_pt(a, g, i, j); });
    else blk_colour(a, 1, [&](int i, int j) { adj_gather_pt(a, g, i, j, -1.0); });
  }
}

template <int DIM>
__device__ void blk_adj_prolong(const Lvl<double>& f, const AdjLvl& gf, const Lvl<double>& c, const AdjLvl& gc,
                                int diag) {
  const int nx = c.mx + 3, ny = c.my + 3, nz = DIM == 3 ? c.mz + 3 : 1, n = nx * ny * nz;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int I = t % nx, J = (t / nx) % ny, K = t / (nx * ny);
    if (DIM == 3) adj_prolong_pt3(f, gf, c, gc, diag, K, J, I);
    else adj_prolong_pt(f, gf, c, gc, diag, J, I);
  }
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

template <int DIM>
__global__ void __launch_bounds__(1024) k_adj_seg_fwd(const AdjTables* tabs, const AdjSeg* seg, int snapshots,
                                                     int diag) {
  __shared__ AdjSegStage st;
  stage_seg(&st, tabs, seg);
  for (int o = 0; o < st.seg.n; ++o) {
    const AdjSegOp op = st.seg.op[o];
    const Lvl<double>& a = st.tab.lv.l[op.lev];
    if (op.kind == kAdjOpRestrict) {
      blk_restrict<double, DIM>(a, st.tab.lv.l[op.lev + 1]);
      continue;
    }
    if (op.kind == kAdjOpSweep) blk_sweep<double, DIM>(a);
    else blk_prolong<double, DIM>(a, st.tab.lv.l[op.lev + 1], diag != 0);
    if (snapshots) {
      const long long n = DIM == 3 ? a.S * (a.mz + 3) : (long long)a.P * (a.my + 3);
      for (long long t = threadIdx.x; t < n; t += blockDim.x) op.after[t] = a.phi[t];
      __syncthreads();
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(1024) k_adj_seg_rev(const AdjTables* tabs, const AdjSeg* seg, int diag) {
  __shared__ AdjSegStage st;
  stage_seg(&st, tabs, seg);
  for (int o = st.seg.n - 1; o >= 0; --o) {
    const AdjSegOp op = st.seg.op[o];
    const Lvl<double>& a = st.tab.lv.l[op.lev];
    const AdjLvl& g = st.tab.g[op.lev];
    if (op.kind == kAdjOpSweep) blk_adj_sweep<DIM>(a, g, op.before, op.after);
    else if (op.kind == kAdjOpProlong)
      blk_adj_prolong<DIM>(a, g, st.tab.lv.l[op.lev + 1], st.tab.g[op.lev + 1], diag);
    else blk_adj_restrict<DIM>(a, g, op.before, st.tab.lv.l[op.lev + 1], st.tab.g[op.lev + 1]);
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
void adj_seg_fwd(int dim, const AdjTables* t, const AdjSeg* g, bool snapshots, int diag, cudaStream_t s) {
  if (dim == 3) k_adj_seg_fwd<3><<<1, 1024, 0, s>>>(t, g, snapshots ? 1 : 0, diag);
  else k_adj_seg_fwd<2><<<1, 1024, 0, s>>>(t, g, snapshots ? 1 : 0, diag);
}
void adj_seg_rev(int dim, const AdjTables* t, const AdjSeg* g, int diag, cudaStream_t s) {
  if (dim == 3) k_adj_seg_rev<3><<<1, 1024, 0, s>>>(t, g, diag);
  else k_adj_seg_rev<2><<<1, 1024, 0, s>>>(t, g, diag);
}

}  // namespace jmg
