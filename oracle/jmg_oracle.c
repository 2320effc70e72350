/*
 * jmg_oracle.c — CPU oracle (test infrastructure only): C/OpenMP restatement of
 * davef96/jsolver's multigrid solve, used as the checker of the CUDA solver and as the
 * timed multi-core CPU baseline. The product library never links or calls it.
 *
 * Same algorithm, same arithmetic order, true division by A_cc as in the reference
 * (compiled with -ffp-contract=off so no multiply-add is fused):
 *   coefficient hierarchy ..... solver_2d.py:326-421, solver_3d.py:338-429
 *   red-black Gauss-Seidel .... solver_2d.py:670-692, solver_3d.py:679-706
 *   defect + restriction ...... solver_2d.py:616-647, solver_3d.py:622-652
 *   prolongation .............. solver_2d.py:649-668, solver_3d.py:654-677
 *   cycle recursion ........... solver_2d.py:582-614, solver_3d.py:588-620
 *   driver .................... solver_2d.py:423-479, solver_3d.py:431-486
 * Arrays use the reference's dense padded layout ((m+3)^d, row-major [z][y][x]).
 * The stencil is stored as face couplings wx/wy/wz plus the diagonal cc (the values of
 * the reference's AMat_* arrays: A_lc(p) = wx[p-1], A_rc(p) = wx[p], etc.).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int m[3];
  int nx, ny, nz;
  long sy, sz; /* strides */
  long n;
  double *phi, *rhs, *wx, *wy, *wz, *cc;
  double *d[3]; /* 3D averaged D of this level (levels >= 1) */
} Level;

typedef struct {
  int dim, L, used;
  int gamma, fcycle, nu1, nu2, diag;
  Level lv[24];
} Ctx;

static inline long IX(const Level* a, int k, int j, int i) { return (long)k * a->sz + (long)j * a->sy + i; }

/* ---- hierarchy ------------------------------------------------------------------ */

static double raw2d(const Ctx* c, const double* D0, int l, int J, int I) {
  const Level* a = &c->lv[l];
  const Level* b = &c->lv[0];
  if (l == 0) return D0[(long)J * b->sy + I];
  if (J < 1 || J > a->m[1] + 1 || I < 1 || I > a->m[0] + 1) return 0.0;
  const int FJ = ((J - 1) << l) + 1, FI = ((I - 1) << l) + 1;
  return D0[(long)FJ * b->sy + FI];
}

static double lam_at(const Ctx* c, const double* lam, double lam_s, int l, int K, int J, int I) {
  if (!lam) return lam_s;
  const Level* b = &c->lv[0];
  if (l == 0) return lam[IX(b, K, J, I)];
  const int FK = c->dim == 3 ? ((K - 1) << l) + 1 : 0;
  return lam[IX(b, FK, ((J - 1) << l) + 1, ((I - 1) << l) + 1)];
}

static double pre3d(const Ctx* c, const double* D0, int comp, int l, int K, int J, int I) {
  const Level* a = &c->lv[l];
  if (K < 1 || K > a->m[2] + 1 || J < 1 || J > a->m[1] + 1 || I < 1 || I > a->m[0] + 1) return 0.0;
  const int k = 2 * K - 1, j = 2 * J - 1, i = 2 * I - 1;
  if (l == 1) return D0[IX(&c->lv[0], k, j, i)];
  const Level* p = &c->lv[l - 1];
  return p->d[comp][IX(p, k, j, i)];
}

static void build_level(Ctx* c, int l, const double* const* D, const double* Ds, int scalarD, const double* lam,
                        double lam_s, const double* sq) {
  Level* a = &c->lv[l];
  const int nx = a->nx, ny = a->ny, nz = a->nz, mx = a->m[0], my = a->m[1], mz = a->m[2];
#pragma omp parallel for collapse(2) schedule(static)
  for (int K = 0; K < nz; ++K)
    for (int J = 0; J < ny; ++J)
      for (int I = 0; I < nx; ++I) {
        const long p = IX(a, K, J, I);
        double w[3] = {0, 0, 0};
        if (scalarD) {
          for (int q = 0; q < c->dim; ++q) w[q] = Ds[q] * sq[q];
        } else if (c->dim == 2) {
          if (J >= 1 && J <= my + 1 && I <= mx + 1) w[0] = (0.5 * (raw2d(c, D[0], l, J, I + 1) + raw2d(c, D[0], l, J, I))) * sq[0];
          if (J <= my + 1 && I >= 1 && I <= mx + 1) w[1] = (0.5 * (raw2d(c, D[1], l, J + 1, I) + raw2d(c, D[1], l, J, I))) * sq[1];
        } else if (l == 0) {
          for (int q = 0; q < 3; ++q) w[q] = D[q][p] * sq[q];
        } else {
          const int iK = K >= 1 && K <= mz + 1, iJ = J >= 1 && J <= my + 1, iI = I >= 1 && I <= mx + 1;
          double dd[3];
          dd[0] = (iK && iJ && I <= mx + 1) ? 0.5 * (pre3d(c, D[0], 0, l, K, J, I + 1) + pre3d(c, D[0], 0, l, K, J, I))
                                           : pre3d(c, D[0], 0, l, K, J, I);
          dd[1] = (iK && J <= my + 1 && iI) ? 0.5 * (pre3d(c, D[1], 1, l, K, J + 1, I) + pre3d(c, D[1], 1, l, K, J, I))
                                           : pre3d(c, D[1], 1, l, K, J, I);
          dd[2] = (K <= mz + 1 && iJ && iI) ? 0.5 * (pre3d(c, D[2], 2, l, K + 1, J, I) + pre3d(c, D[2], 2, l, K, J, I))
                                           : pre3d(c, D[2], 2, l, K, J, I);
          for (int q = 0; q < 3; ++q) {
            a->d[q][p] = dd[q];
            w[q] = dd[q] * sq[q];
          }
        }
        a->wx[p] = w[0];
        a->wy[p] = w[1];
        if (c->dim == 3) a->wz[p] = w[2];
      }
#pragma omp parallel for collapse(2) schedule(static)
  for (int K = 0; K < nz; ++K)
    for (int J = 0; J < ny; ++J)
      for (int I = 0; I < nx; ++I) {
        const long p = IX(a, K, J, I);
        const int in = J >= 2 && J <= my && I >= 2 && I <= mx && (c->dim == 2 || (K >= 2 && K <= mz));
        double acc = 0.0;
        if (in) {
          const double lm = lam_at(c, lam, lam_s, l, K, J, I);
          if (scalarD) {
            double s = Ds[0] * sq[0] + Ds[1] * sq[1];
            if (c->dim == 3) s = s + Ds[2] * sq[2];
            acc = 2.0 * s + lm;
          } else {
            double s = a->wx[p - 1] + a->wx[p];
            s = s + a->wy[p - a->sy];
            s = s + a->wy[p];
            if (c->dim == 3) {
              s = s + a->wz[p - a->sz];
              s = s + a->wz[p];
            }
            acc = s + lm;
          }
        }
        a->cc[p] = acc;
      }
}

/* ---- operators ------------------------------------------------------------------- */

static inline double defect_at(const Ctx* c, const Level* a, long p) {
  const long sy = a->sy, sz = a->sz;
  double d = a->cc[p] * a->phi[p] - a->wx[p - 1] * a->phi[p - 1] - a->wx[p] * a->phi[p + 1] -
             a->wy[p - sy] * a->phi[p - sy] - a->wy[p] * a->phi[p + sy];
  if (c->dim == 3) d = d - a->wz[p - sz] * a->phi[p - sz] - a->wz[p] * a->phi[p + sz];
  return d + a->rhs[p];
}

static void sweep(const Ctx* c, Level* a) {
  const long sy = a->sy, sz = a->sz;
  const int mx = a->m[0], my = a->m[1], mz = c->dim == 3 ? a->m[2] : 2;
  for (int color = 0; color < 2; ++color) {
    /* first colour: i+j even in 2D (sub-lattices (0,0),(1,1)); i+j+k odd in 3D */
    const int par = c->dim == 2 ? color : (1 + color) & 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 2; k <= mz; ++k)
      for (int j = 2; j <= my; ++j) {
        const int kk = c->dim == 3 ? k : 0;
        const int i0 = 2 + ((j + kk + par) & 1);
        for (int i = i0; i <= mx; i += 2) {
          const long p = IX(a, kk, j, i);
          double s;
          if (c->dim == 2) {
            s = a->wy[p] * a->phi[p + sy] + a->wy[p - sy] * a->phi[p - sy] + a->wx[p] * a->phi[p + 1] +
                a->wx[p - 1] * a->phi[p - 1] - a->rhs[p];
          } else {
            s = a->wz[p] * a->phi[p + sz] + a->wz[p - sz] * a->phi[p - sz] + a->wy[p] * a->phi[p + sy] +
                a->wy[p - sy] * a->phi[p - sy] + a->wx[p] * a->phi[p + 1] + a->wx[p - 1] * a->phi[p - 1] - a->rhs[p];
          }
          a->phi[p] = s / a->cc[p];
        }
      }
  }
}

static void restrict_to(const Ctx* c, const Level* f, Level* q) {
  memset(q->phi, 0, sizeof(double) * q->n);
  memset(q->rhs, 0, sizeof(double) * q->n);
  const int mx = q->m[0], my = q->m[1], mz = c->dim == 3 ? q->m[2] : 2;
  const long sy = f->sy, sz = f->sz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int K = 2; K <= mz; ++K)
    for (int J = 2; J <= my; ++J)
      for (int I = 2; I <= mx; ++I) {
        if (c->dim == 2) {
          const long ctr = IX(f, 0, 2 * J - 1, 2 * I - 1);
          double s = defect_at(c, f, ctr + sy + 1) + defect_at(c, f, ctr + sy - 1);
          s = s + defect_at(c, f, ctr - sy + 1);
          s = s + defect_at(c, f, ctr - sy - 1);
          q->rhs[IX(q, 0, J, I)] = 0.0625 * s + 0.25 * defect_at(c, f, ctr);
        } else {
          const long ctr = IX(f, 2 * K - 1, 2 * J - 1, 2 * I - 1);
          const long off[12] = {sy + 1, sy - 1, -sy + 1, -sy - 1, sz + 1, sz - 1,
                                -sz + 1, -sz - 1, sz + sy, sz - sy, -sz + sy, -sz - sy};
          double s = defect_at(c, f, ctr + off[0]);
          for (int t = 1; t < 12; ++t) s = s + defect_at(c, f, ctr + off[t]);
          q->rhs[IX(q, K, J, I)] = 0.03125 * s + 0.125 * defect_at(c, f, ctr);
        }
      }
}

static void prolong_add(const Ctx* c, Level* f, const Level* q) {
  const int mx = f->m[0], my = f->m[1], mz = c->dim == 3 ? f->m[2] : 2;
  const double* pc = q->phi;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 2; k <= mz; ++k)
    for (int j = 2; j <= my; ++j)
      for (int i = 2; i <= mx; ++i) {
        const int kk = c->dim == 3 ? k : 1; /* 2D: treat k as odd so it never counts as even */
        const int ke = c->dim == 3 ? !(kk & 1) : 0, je = !(j & 1), ie = !(i & 1);
        const int ne = ke + je + ie;
        const int kp = ke ? (kk + 2) / 2 : (kk + 1) / 2, km = ke ? kk / 2 : kp;
        const int jp = je ? (j + 2) / 2 : (j + 1) / 2, jm = je ? j / 2 : jp;
        const int ip = ie ? (i + 2) / 2 : (i + 1) / 2, im = ie ? i / 2 : ip;
        const int K0 = c->dim == 3 ? kp : 0, K1 = c->dim == 3 ? km : 0;
#define C3(a, b, d) pc[IX(q, a, b, d)]
        double v;
        if (ne == 0) v = C3(K0, jp, ip);
        else if (ne == 1) {
          if (ie) v = 0.5 * (C3(K0, jp, ip) + C3(K0, jp, im));
          else if (je) v = 0.5 * (C3(K0, jp, ip) + C3(K0, jm, ip));
          else v = 0.5 * (C3(K0, jp, ip) + C3(K1, jp, ip));
        } else if (ne == 2) {
          if (!c->diag) continue;
          if (!ke) v = 0.25 * (C3(K0, jp, ip) + C3(K0, jm, ip) + C3(K0, jp, im) + C3(K0, jm, im));
          else if (!je) v = 0.25 * (C3(K0, jp, ip) + C3(K1, jp, ip) + C3(K0, jp, im) + C3(K1, jp, im));
          else v = 0.25 * (C3(K0, jp, ip) + C3(K1, jp, ip) + C3(K0, jm, ip) + C3(K1, jm, ip));
        } else {
          v = 0.125 * (C3(K0, jp, ip) + C3(K1, jp, ip) + C3(K0, jm, ip) + C3(K1, jm, ip) + C3(K0, jp, im) +
                       C3(K1, jp, im) + C3(K0, jm, im) + C3(K1, jm, im));
        }
#undef C3
        const long p = IX(f, c->dim == 3 ? k : 0, j, i);
        f->phi[p] = f->phi[p] + v;
      }
}

static void cycle(Ctx* c, int l, int fcycle, int skip_pre) {
  Level* a = &c->lv[l];
  if (l == c->L - 2) {
    for (int s = 0; s < c->nu1 + c->nu2; ++s) sweep(c, a);
    return;
  }
  if (!skip_pre)
    for (int s = 0; s < c->nu1; ++s) sweep(c, a);
  restrict_to(c, a, &c->lv[l + 1]);
  if (fcycle)
    for (int g = 0; g < c->gamma; ++g) cycle(c, l + 1, 1, 0);
  for (int g = 0; g < c->gamma; ++g) cycle(c, l + 1, 0, 0);
  prolong_add(c, a, &c->lv[l + 1]);
  for (int s = 0; s < c->nu2; ++s) sweep(c, a);
}

static void zero_frame(const Ctx* c, Level* a) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int K = 0; K < a->nz; ++K)
    for (int J = 0; J < a->ny; ++J)
      for (int I = 0; I < a->nx; ++I) {
        const int fr = I < 2 || I >= a->nx - 2 || J < 2 || J >= a->ny - 2 || (c->dim == 3 && (K < 2 || K >= a->nz - 2));
        if (fr) a->phi[IX(a, K, J, I)] = 0.0;
      }
}

static double residual_norm(const Ctx* c, const Level* a, int use_phi) {
  const int mx = a->m[0], my = a->m[1], mz = c->dim == 3 ? a->m[2] : 2;
  double s = 0.0;
#pragma omp parallel for collapse(2) reduction(+ : s) schedule(static)
  for (int k = 2; k <= mz; ++k)
    for (int j = 2; j <= my; ++j)
      for (int i = 2; i <= mx; ++i) {
        const long p = IX(a, c->dim == 3 ? k : 0, j, i);
        const double d = use_phi ? defect_at(c, a, p) : a->rhs[p];
        s += d * d;
      }
  return sqrt(s);
}

/* ---- public entry ----------------------------------------------------------------- */

static void free_ctx(Ctx* c) {
  for (int l = 0; l < c->used; ++l) {
    Level* a = &c->lv[l];
    free(a->phi); free(a->rhs); free(a->wx); free(a->wy); free(a->wz); free(a->cc);
    for (int q = 0; q < 3; ++q) free(a->d[q]);
  }
}

/* Returns the cycle count (>= 0), or -1 on bad arguments. rel_res_out (optional)
 * receives the final relative residual. stop: 0 distance, 1 relative residual. */
int64_t jmgo_solve(int dim, const int32_t* m, const double* idel, const double* phi0, const double* rhs,
                   const double* lam, double lam_s, const double* const* D, const double* Ds, int fixed,
                   double eps, int gamma, int fcycle, int skip_pre, int nu1, int nu2, int64_t max_iters, int stop,
                   double rtol, double* phi_out, double* rel_res_out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  Ctx c;
  memset(&c, 0, sizeof(c));
  c.dim = dim;
  int L = 1 << 30;
  for (int a = 0; a < dim; ++a) {
    int lv = (int)ceil(log2((double)m[a])) + 1;
    if (lv < L) L = lv;
  }
  if (L < 2 || L > 24) return -1;
  c.L = L;
  c.used = L - 1;
  c.gamma = gamma > 0 ? gamma : 0;
  c.fcycle = fcycle;
  c.nu1 = nu1 > 0 ? nu1 : 0;
  c.nu2 = nu2 > 0 ? nu2 : 0;
  c.diag = nu2 <= 0;
  int scalarD = 1;
  for (int a = 0; a < dim; ++a)
    if (D[a]) scalarD = 0;
  for (int l = 0; l < c.used; ++l) {
    Level* a = &c.lv[l];
    for (int q = 0; q < 3; ++q) a->m[q] = q < dim ? (m[q] >> l) : 0;
    a->nx = a->m[0] + 3;
    a->ny = a->m[1] + 3;
    a->nz = dim == 3 ? a->m[2] + 3 : 1;
    a->sy = a->nx;
    a->sz = (long)a->nx * a->ny;
    a->n = a->sz * a->nz;
    a->phi = calloc(a->n, 8);
    a->rhs = calloc(a->n, 8);
    a->wx = calloc(a->n, 8);
    a->wy = calloc(a->n, 8);
    a->wz = dim == 3 ? calloc(a->n, 8) : NULL;
    a->cc = calloc(a->n, 8);
    for (int q = 0; q < 3; ++q) a->d[q] = (dim == 3 && l >= 1) ? calloc(a->n, 8) : NULL;
  }
  for (int l = 0; l < c.used; ++l) {
    double sq[3] = {0, 0, 0};
    for (int q = 0; q < dim; ++q) {
      const double id = idel[q] * pow(0.5, l);
      sq[q] = id * id;
    }
    build_level(&c, l, D, Ds, scalarD, lam, lam_s, sq);
  }
  Level* a0 = &c.lv[0];
  memcpy(a0->phi, phi0, a0->n * 8);
  memcpy(a0->rhs, rhs, a0->n * 8);
  double* old = malloc(a0->n * 8);
  const double rhs_norm = residual_norm(&c, a0, 0);
  if (skip_pre) {
    zero_frame(&c, a0);
    for (int s = 0; s < c.nu1; ++s) sweep(&c, a0);
  }
  int64_t count = 0;
  if (fixed) {
    for (int64_t it = 0; it < max_iters; ++it) {
      zero_frame(&c, a0);
      cycle(&c, 0, fcycle, skip_pre);
    }
    count = max_iters;
  } else {
    double crit = INFINITY;
    if (stop == 1) crit = residual_norm(&c, a0, 1) / rhs_norm;
    const double tol = stop == 1 ? rtol : eps;
    while (crit > tol && count < max_iters) {
      memcpy(old, a0->phi, a0->n * 8);
      zero_frame(&c, a0);
      cycle(&c, 0, fcycle, skip_pre);
      ++count;
      if (stop == 1) {
        crit = residual_norm(&c, a0, 1) / rhs_norm;
      } else {
        double mx = 0.0;
        int nan = 0;
#pragma omp parallel for reduction(max : mx) reduction(| : nan) schedule(static)
        for (long p = 0; p < a0->n; ++p) {
          const double d = fabs(old[p] - a0->phi[p]);
          if (d != d) nan = 1;
          else if (d > mx) mx = d;
        }
        crit = nan ? NAN : mx;
      }
    }
  }
  if (rel_res_out) *rel_res_out = residual_norm(&c, a0, 1) / rhs_norm;
  memcpy(phi_out, a0->phi, a0->n * 8);
  free(old);
  free_ctx(&c);
  return count;
}

/* Time-bounded sample: runs `cycles` V/W/F cycles from phi0 (no stopping test) and
 * returns the relative residual; used to scale per-cycle CPU time for the baseline. */
double jmgo_cycles(int dim, const int32_t* m, const double* idel, const double* phi0, const double* rhs,
                   const double* lam, double lam_s, const double* const* D, const double* Ds, int gamma, int fcycle,
                   int nu1, int nu2, int64_t cycles, double* phi_out, int nthreads) {
  double rr = 0.0;
  jmgo_solve(dim, m, idel, phi0, rhs, lam, lam_s, D, Ds, 1, 0.0, gamma, fcycle, 0, nu1, nu2, cycles, 0, 0.0,
             phi_out, &rr, nthreads);
  return rr;
}

int jmgo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
