// mg_hierarchy.cu — per-level stencil coefficients, built on the device once per solve.
//
// Follows the reference bit for bit (same operations, same order, no contraction):
//  2D (solver_2d.py:326-421): D is injected *raw* to every level, D_l[J,I] =
//     D_0[F(J), F(I)] with F(K) = 2^l (K-1) + 1 on J, I in 1..m_l+1 and 0 on the rest of
//     the ring (lines 352-356); then every level, level 0 included, is face-averaged,
//     Dx[J, I] = 0.5 (D[J, I+1] + D[J, I]) on J in 1..m+1, I in 0..m+1 (lines 359-361).
//  3D (solver_3d.py:338-429): level 0 keeps the raw cell values; level l >= 1 injects
//     from level l-1 (already averaged when l-1 >= 1) and then averages (lines 363-370).
//     The averaged coarse arrays are therefore kept in the workspace for the next level.
//  lambda (solver_2d.py:365-383; solver_3d.py:374-392) is injected: lam_l = lam_0[F(.)].
//  A_cc = A_lc + A_rc + A_cl + A_cr (+ z) + lam (solver_2d.py:409; solver_3d.py:422);
//  scalar D: A_cc = 2 (A_x + A_y (+ A_z)) + lam (solver_2d.py:418-421; solver_3d.py:425-429).
// invd = 1 / A_cc is the only value the reference does not form: it divides by A_cc in
// every sweep (solver_2d.py:687); multiplying by a correctly rounded reciprocal differs
// from that division by at most one rounding.
#include "mg_kernels.h"

namespace jmg {

struct HierArgs {
  Lvl<double> a;   // this level's output arrays
  Box b;           // this level's padded box
  Box b0;          // level-0 box (user arrays are dense with pitch b0.nx)
  Box bp;          // previous level's box (3D averaged arrays)
  int level, dim;
  int scalar_D, scalar_lam;
  const double* D[3];
  double Ds[3];
  const double* lam;
  double lam_s;
  double sq[3];    // idel_l^2 per axis
  double cxy;      // 2D with D_xy: idel_x,l * idel_y,l * 0.25 (solver_2d.py:410)
  double* dcur[3];        // 3D: averaged D of this level (level >= 1)
  const double* dprev[3]; // 3D: averaged D of level-1 (level-1 >= 1)
};

__device__ __forceinline__ long long dense_idx(const Box& b0, int K, int J, int I) {
  return ((long long)K * b0.ny + J) * b0.nx + I;
}

// F^l(K): fine index of coarse index K after l injections (K in 1..m_l+1)
__device__ __forceinline__ int finer(int K, int level) { return ((K - 1) << level) + 1; }

__device__ __forceinline__ double lam_at(const HierArgs& h, int K, int J, int I) {
  if (h.scalar_lam) return h.lam_s;
  if (h.level == 0) return h.lam[dense_idx(h.b0, K, J, I)];
  return h.lam[dense_idx(h.b0, h.dim == 3 ? finer(K, h.level) : 0, finer(J, h.level), finer(I, h.level))];
}

// 2D raw injected D of component c at level l (index (J, I) of the padded box)
__device__ __forceinline__ double raw2d(const HierArgs& h, int c, int J, int I) {
  if (h.level == 0) return h.D[c][dense_idx(h.b0, 0, J, I)];
  const int my = h.b.ny - 3, mx = h.b.nx - 3;
  if (J < 1 || J > my + 1 || I < 1 || I > mx + 1) return 0.0;
  return h.D[c][dense_idx(h.b0, 0, finer(J, h.level), finer(I, h.level))];
}

__global__ void k_hier_faces2d(HierArgs h) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= h.b.nx || J >= h.b.ny) return;
  const int mx = h.b.nx - 3, my = h.b.ny - 3;
  const long long p = (long long)J * h.b.P + I;
  double wx = 0.0, wy = 0.0;
  if (h.scalar_D) {
    wx = h.Ds[0] * h.sq[0];
    wy = h.Ds[1] * h.sq[1];
  } else {
    if (J >= 1 && J <= my + 1 && I <= mx + 1) {
      const double avg = 0.5 * __dadd_rn(raw2d(h, 0, J, I + 1), raw2d(h, 0, J, I));
      wx = __dmul_rn(avg, h.sq[0]);
    }
    if (J <= my + 1 && I >= 1 && I <= mx + 1) {
      const double avg = 0.5 * __dadd_rn(raw2d(h, 1, J + 1, I), raw2d(h, 1, J, I));
      wy = __dmul_rn(avg, h.sq[1]);
    }
  }
  h.a.wx[p] = wx;
  h.a.wy[p] = wy;
}

__global__ void k_hier_diag2d(HierArgs h) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= h.b.nx || J >= h.b.ny) return;
  const int mx = h.b.nx - 3, my = h.b.ny - 3;
  const long long p = (long long)J * h.b.P + I;
  double acc = 0.0, inv = 0.0;
  if (J >= 2 && J <= my && I >= 2 && I <= mx) {
    const double lam = lam_at(h, 0, J, I);
    if (h.scalar_D) {
      const double add = 2.0 * __dadd_rn(__dmul_rn(h.Ds[0], h.sq[0]), __dmul_rn(h.Ds[1], h.sq[1]));
      acc = __dadd_rn(add, lam);
    } else {
      const double* wx = h.a.wx;
      const double* wy = h.a.wy;
      const int P = h.b.P;
      double s = __dadd_rn(wx[p - 1], wx[p]);
      s = __dadd_rn(s, wy[p - P]);
      s = __dadd_rn(s, wy[p]);
      acc = __dadd_rn(s, lam);
    }
    inv = 1.0 / acc;
  }
  h.a.acc[p] = acc;
  h.a.invd[p] = inv;
}

// 2D with D_xy: the diagonal couplings of level l from the raw injected D_xy (no face
// averaging for D_xy), on J, I in 1..m+1 (solver_2d.py:352-356, 410-416):
//   A_ll = (Dxy[J][I-1] + Dxy[J-1][I]) c      A_lr = -(Dxy[J][I-1] + Dxy[J+1][I]) c
//   A_rl = -(Dxy[J][I+1] + Dxy[J-1][I]) c     A_rr = (Dxy[J][I+1] + Dxy[J+1][I]) c
// with c = idel_x * idel_y * 0.25 and D_xy in slot 2 of h.D.
__global__ void k_hier_xy2d(HierArgs h) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= h.b.nx || J >= h.b.ny) return;
  const int mx = h.b.nx - 3, my = h.b.ny - 3;
  const long long p = (long long)J * h.b.P + I;
  double ll = 0.0, lr = 0.0, rl = 0.0, rr = 0.0;
  if (J >= 1 && J <= my + 1 && I >= 1 && I <= mx + 1) {
    const double w = raw2d(h, 2, J, I - 1), e = raw2d(h, 2, J, I + 1);
    const double sth = raw2d(h, 2, J - 1, I), nth = raw2d(h, 2, J + 1, I);
    ll = __dmul_rn(__dadd_rn(w, sth), h.cxy);
    lr = __dmul_rn(-__dadd_rn(w, nth), h.cxy);
    rl = __dmul_rn(-__dadd_rn(e, sth), h.cxy);
    rr = __dmul_rn(__dadd_rn(e, nth), h.cxy);
  }
  h.a.xll[p] = ll;
  h.a.xlr[p] = lr;
  h.a.xrl[p] = rl;
  h.a.xrr[p] = rr;
}

// 3D: source of level l's injection for component c at coarse (K, J, I) in 1..m+1
__device__ __forceinline__ double pre3d(const HierArgs& h, int c, int K, int J, int I) {
  const int mx = h.b.nx - 3, my = h.b.ny - 3, mz = h.b.nz - 3;
  if (K < 1 || K > mz + 1 || J < 1 || J > my + 1 || I < 1 || I > mx + 1) return 0.0;
  const int k = 2 * K - 1, j = 2 * J - 1, i = 2 * I - 1;
  if (h.level == 1) return h.D[c][dense_idx(h.b0, k, j, i)];
  return h.dprev[c][(long long)k * h.bp.S + (long long)j * h.bp.P + i];
}

__global__ void k_hier_faces3d(HierArgs h) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= h.b.nx || J >= h.b.ny) return;
  const int mx = h.b.nx - 3, my = h.b.ny - 3, mz = h.b.nz - 3;
  const long long p = (long long)K * h.b.S + (long long)J * h.b.P + I;
  double w[3];
  if (h.scalar_D) {
    for (int c = 0; c < 3; ++c) w[c] = h.Ds[c] * h.sq[c];
  } else if (h.level == 0) {
    const long long q = dense_idx(h.b0, K, J, I);
    for (int c = 0; c < 3; ++c) w[c] = __dmul_rn(h.D[c][q], h.sq[c]);
  } else {
    const bool inK = K >= 1 && K <= mz + 1, inJ = J >= 1 && J <= my + 1, inI = I >= 1 && I <= mx + 1;
    double d[3];
    d[0] = (inK && inJ && I <= mx + 1) ? 0.5 * __dadd_rn(pre3d(h, 0, K, J, I + 1), pre3d(h, 0, K, J, I))
                                       : pre3d(h, 0, K, J, I);
    d[1] = (inK && J <= my + 1 && inI) ? 0.5 * __dadd_rn(pre3d(h, 1, K, J + 1, I), pre3d(h, 1, K, J, I))
                                       : pre3d(h, 1, K, J, I);
    d[2] = (K <= mz + 1 && inJ && inI) ? 0.5 * __dadd_rn(pre3d(h, 2, K + 1, J, I), pre3d(h, 2, K, J, I))
                                       : pre3d(h, 2, K, J, I);
    for (int c = 0; c < 3; ++c) {
      h.dcur[c][p] = d[c];
      w[c] = __dmul_rn(d[c], h.sq[c]);
    }
  }
  h.a.wx[p] = w[0];
  h.a.wy[p] = w[1];
  h.a.wz[p] = w[2];
}

__global__ void k_hier_diag3d(HierArgs h) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= h.b.nx || J >= h.b.ny) return;
  const int mx = h.b.nx - 3, my = h.b.ny - 3, mz = h.b.nz - 3;
  const long long p = (long long)K * h.b.S + (long long)J * h.b.P + I;
  double acc = 0.0, inv = 0.0;
  if (K >= 2 && K <= mz && J >= 2 && J <= my && I >= 2 && I <= mx) {
    const double lam = lam_at(h, K, J, I);
    if (h.scalar_D) {
      double s = __dadd_rn(__dmul_rn(h.Ds[0], h.sq[0]), __dmul_rn(h.Ds[1], h.sq[1]));
      s = __dadd_rn(s, __dmul_rn(h.Ds[2], h.sq[2]));
      acc = __dadd_rn(2.0 * s, lam);
    } else {
      const double *wx = h.a.wx, *wy = h.a.wy, *wz = h.a.wz;
      const int P = h.b.P;
      const long long S = h.b.S;
      double s = __dadd_rn(wx[p - 1], wx[p]);
      s = __dadd_rn(s, wy[p - P]);
      s = __dadd_rn(s, wy[p]);
      s = __dadd_rn(s, wz[p - S]);
      s = __dadd_rn(s, wz[p]);
      acc = __dadd_rn(s, lam);
    }
    inv = 1.0 / acc;
  }
  h.a.acc[p] = acc;
  h.a.invd[p] = inv;
}

static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

void launch_hierarchy_level(int dim, int level, const Lvl<double>& a, const Box& b, const Box& b0,
                            const HierInputs& in, const double* idel, const double* sq_idel, double* const* d_cur,
                            const double* const* d_prev, const Box& bprev, cudaStream_t s) {
  HierArgs h;
  h.a = a;
  h.b = b;
  h.b0 = b0;
  h.bp = bprev;
  h.level = level;
  h.dim = dim;
  h.scalar_D = in.scalar_D;
  h.scalar_lam = in.scalar_lam;
  for (int c = 0; c < 3; ++c) {
    h.D[c] = in.D[c];
    h.Ds[c] = in.D_scalar[c];
    h.sq[c] = sq_idel[c];
    h.dcur[c] = d_cur ? d_cur[c] : nullptr;
    h.dprev[c] = d_prev ? d_prev[c] : nullptr;
  }
  h.lam = in.lam;
  h.lam_s = in.lam_scalar;
  h.cxy = 0.0;
  dim3 blk(32, 8, 1), grd(cdiv(b.nx, 32), cdiv(b.ny, 8), dim == 3 ? b.nz : 1);
  if (dim == 2) {
    k_hier_faces2d<<<grd, blk, 0, s>>>(h);
    k_hier_diag2d<<<grd, blk, 0, s>>>(h);
    if (a.xll && in.Dxy) {
      h.D[2] = in.Dxy;
      h.cxy = (idel[0] * idel[1]) * 0.25;
      k_hier_xy2d<<<grd, blk, 0, s>>>(h);
    }
  } else {
    k_hier_faces3d<<<grd, blk, 0, s>>>(h);
    k_hier_diag3d<<<grd, blk, 0, s>>>(h);
  }
}

}  // namespace jmg
