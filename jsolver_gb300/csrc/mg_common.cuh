// mg_common.cuh — level descriptors and per-point stencil arithmetic of the solver.
//
// Internal layout in the workspace: every level l keeps its padded arrays
// ((m_y+3) x (m_x+3) in 2D, (m_z+3) x (m_y+3) x (m_x+3) in 3D, the reference's shapes,
// solver_2d.py:302 / solver_3d.py:310) with a row pitch P rounded up to 16 elements, so
// that rows start on 128-byte boundaries, and plane stride S = P * (m_y+3).
//
// Coefficients are stored as face arrays plus the diagonal, which is the reference's
// AMat_* set (solver_2d.py:403-409; solver_3d.py:413-422) without duplication:
//   wx[p] = coupling between p and p+1 (x),  A_lc(p) = wx[p-1], A_rc(p) = wx[p]
//   wy[p] = coupling between p and p+P (y),  A_cl(p) = wy[p-P], A_cr(p) = wy[p]
//   wz[p] = coupling between p and p+S (z),  A_ccl(p) = wz[p-S], A_ccr(p) = wz[p]
//   acc[p] = A_cc(p), invd[p] = 1 / A_cc(p)
// Interior unknowns are indices 2..m on every axis; the frame {0, 1, m+1, m+2} is zero
// in phi and rhs at all times (do_BCs, boundary_handler_2d.py:21-30).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace jmg {

template <typename T>
struct Lvl {
  T* phi;
  T* rhs;
  T* wx;
  T* wy;
  T* wz;
  T* invd;
  T* acc;
  // 2D with D_xy (9-point stencil): diagonal couplings of p with its SW, SE, NW and NE
  // neighbours, the reference's A_ll, A_rl, A_lr, A_rr (solver_2d.py:410-416); nullptr
  // without D_xy
  T* xll;
  T* xrl;
  T* xlr;
  T* xrr;
  int mx, my, mz;  // resolution per axis (interior indices 2..m)
  int P;           // row pitch in elements
  long long S;     // plane stride in elements (3D)
  // second phi buffer of a level swept in one pass or by the fused operator pairs (those
  // kernels write it and swap the two); nullptr where the level uses in-place passes only
  T* phi2;
  int onepass;  // the level's sweeps run in one pass (needs phi2)
  int fuseops;  // 2D: smooth + restrict and prolong + smooth as fused tile kernels (needs phi2)
};

constexpr int kMaxLevels = 16;

// Programmatic dependent launch (PDL). Kernels of the cycle are launched with
// programmatic stream serialisation (launch_k in mg_kernels.h): the next kernel may be
// scheduled while this one drains. pdl_enter() at the top of a kernel first waits until
// the preceding kernel has completed and its writes are visible (griddepcontrol.wait;
// a no-op without a programmatic dependency), so no data hazard is relaxed, then lets the
// following kernel start launching (griddepcontrol.launch_dependents).
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
#ifdef JMG_PDL_EARLY_TRIGGER
  asm volatile("griddepcontrol.launch_dependents;\n" :::);
#endif
}

template <typename T>
struct LvlTable {
  Lvl<T> l[kMaxLevels];
  // set to 1 by a coarse kernel whose wait for its staging copies ran out (the table is
  // stored afresh, with 0, at every solve)
  int fault;
};

// Red (first) colour of a full sweep. In 2D the reference's first two sub-lattices
// (0,0),(1,1) (solver_2d.py:684) are the points with i+j even; in 3D the first four,
// (0,0,0),(0,1,1),(1,1,0),(1,0,1) (solver_3d.py:693), are the points with i+j+k odd.
// Sub-lattices of one colour never neighbour each other, so updating a colour at
// once is the same arithmetic as the reference's sequence of strided updates.
template <int DIM>
__host__ __device__ constexpr int first_color_parity() { return DIM == 2 ? 0 : 1; }

// ---- 2D -------------------------------------------------------------------------------

// Gauss-Seidel value of one interior point (solver_2d.py:687):
//   (A_cr phi_N + A_cl phi_S + A_rc phi_E + A_lc phi_W - rhs) / A_cc
template <typename T>
__device__ __forceinline__ T gs_point2d(const T* __restrict__ ph, const T* __restrict__ rhs,
                                        const T* __restrict__ wx, const T* __restrict__ wy,
                                        const T* __restrict__ invd, long long p, int P) {
  T s = wy[p] * ph[p + P];
  s = fma(wy[p - P], ph[p - P], s);
  s = fma(wx[p], ph[p + 1], s);
  s = fma(wx[p - 1], ph[p - 1], s);
  s = s - rhs[p];
  return s * invd[p];
}

// Defect rhs - L_h phi at one interior point (solver_2d.py:637):
//   A_cc phi - A_lc phi_W - A_rc phi_E - A_cl phi_S - A_cr phi_N + rhs
template <typename T>
__device__ __forceinline__ T defect_point2d(const T* ph, const T* rhs, const T* __restrict__ wx,
                                            const T* __restrict__ wy, const T* __restrict__ acc,
                                            long long p, int P) {
  T d = acc[p] * ph[p];
  d = fma(-wx[p - 1], ph[p - 1], d);
  d = fma(-wx[p], ph[p + 1], d);
  d = fma(-wy[p - P], ph[p - P], d);
  d = fma(-wy[p], ph[p + P], d);
  return d + rhs[p];
}

// Off-diagonal part of the 9-point stencil at p (D_xy present), in the reference's
// order ((A_ll SW + A_rl SE) + A_lr NW) + A_rr NE (solver_2d.py:686-690, 638-641).
template <typename T>
__device__ __forceinline__ T offdiag2d(const Lvl<T>& a, const T* ph, long long p) {
  const int P = a.P;
  T o = a.xll[p] * ph[p - P - 1];
  o = fma(a.xrl[p], ph[p - P + 1], o);
  o = fma(a.xlr[p], ph[p + P - 1], o);
  o = fma(a.xrr[p], ph[p + P + 1], o);
  return o;
}

// Gauss-Seidel value with the level's full stencil (5-point, or 9-point with D_xy):
// (N/S/E/W part - rhs + off-diagonal part) / A_cc (solver_2d.py:687-690)
template <typename T>
__device__ __forceinline__ T gs_point2d(const Lvl<T>& a, long long p) {
  if (!a.xll) return gs_point2d<T>(a.phi, a.rhs, a.wx, a.wy, a.invd, p, a.P);
  const int P = a.P;
  T s = a.wy[p] * a.phi[p + P];
  s = fma(a.wy[p - P], a.phi[p - P], s);
  s = fma(a.wx[p], a.phi[p + 1], s);
  s = fma(a.wx[p - 1], a.phi[p - 1], s);
  s = s - a.rhs[p];
  s = s + offdiag2d(a, a.phi, p);
  return s * a.invd[p];
}

// Defect of phi (not necessarily a.phi) with the level's full stencil: the 5-point
// defect minus the off-diagonal part (solver_2d.py:637-642).
template <typename T>
__device__ __forceinline__ T defect_point2d(const Lvl<T>& a, const T* ph, long long p) {
  const T d = defect_point2d(ph, a.rhs, a.wx, a.wy, a.acc, p, a.P);
  return a.xll ? d - offdiag2d(a, ph, p) : d;
}

// Coarse right-hand side at coarse interior point (J, I) from the fine defects at the
// red points (solver_2d.py:644): 1/16 of the four diagonal neighbours + 1/4 centre.
template <typename T>
__device__ __forceinline__ T restrict_point2d(const Lvl<T>& f, int J, int I) {
  const int P = f.P;
  const long long c = (long long)(2 * J - 1) * P + (2 * I - 1);
  const T dne = defect_point2d(f, f.phi, c + P + 1);
  const T dnw = defect_point2d(f, f.phi, c + P - 1);
  const T dse = defect_point2d(f, f.phi, c - P + 1);
  const T dsw = defect_point2d(f, f.phi, c - P - 1);
  const T dc = defect_point2d(f, f.phi, c);
  const T s = ((dne + dnw) + dse) + dsw;
  return T(0.0625) * s + T(0.25) * dc;
}

// Prolongated correction at fine interior point (i, j) (solver_2d.py:662-666).
// Returns false for (even, even) points when they are skipped (nu2 > 0, no D_xy).
template <typename T>
__device__ __forceinline__ bool prolong_point2d(const Lvl<T>& c, int i, int j, bool diag, T* out) {
  const T* pc = c.phi;
  const int P = c.P;
  const bool io = i & 1, jo = j & 1;
  if (io && jo) {
    *out = pc[(long long)((i + 1) >> 1) * P + ((j + 1) >> 1)];
  } else if (io) {  // odd row, even column: linear in x
    const long long r = (long long)((i + 1) >> 1) * P;
    *out = T(0.5) * (pc[r + ((j + 2) >> 1)] + pc[r + (j >> 1)]);
  } else if (jo) {  // even row, odd column: linear in y
    const int cj = (j + 1) >> 1;
    *out = T(0.5) * (pc[(long long)((i + 2) >> 1) * P + cj] + pc[(long long)(i >> 1) * P + cj]);
  } else {
    if (!diag) return false;
    const long long rp = (long long)((i + 2) >> 1) * P, rm = (long long)(i >> 1) * P;
    const int cp = (j + 2) >> 1, cm = j >> 1;
    *out = T(0.25) * (((pc[rp + cp] + pc[rm + cp]) + pc[rp + cm]) + pc[rm + cm]);
  }
  return true;
}

// ---- 3D -------------------------------------------------------------------------------

// (A_ccr U + A_ccl D + A_crc N + A_clc S + A_rcc E + A_lcc W - rhs) / A_ccc
// (solver_3d.py:695-698)
template <typename T>
__device__ __forceinline__ T gs_point3d(const T* __restrict__ ph, const T* __restrict__ rhs,
                                        const T* __restrict__ wx, const T* __restrict__ wy,
                                        const T* __restrict__ wz, const T* __restrict__ invd,
                                        long long p, int P, long long S) {
  T s = wz[p] * ph[p + S];
  s = fma(wz[p - S], ph[p - S], s);
  s = fma(wy[p], ph[p + P], s);
  s = fma(wy[p - P], ph[p - P], s);
  s = fma(wx[p], ph[p + 1], s);
  s = fma(wx[p - 1], ph[p - 1], s);
  s = s - rhs[p];
  return s * invd[p];
}

// A_ccc C - A_lcc W - A_rcc E - A_clc S - A_crc N - A_ccl D - A_ccr U + rhs
// (solver_3d.py:642)
template <typename T>
__device__ __forceinline__ T defect_point3d(const T* ph, const T* rhs, const T* __restrict__ wx,
                                            const T* __restrict__ wy, const T* __restrict__ wz,
                                            const T* __restrict__ acc, long long p, int P,
                                            long long S) {
  T d = acc[p] * ph[p];
  d = fma(-wx[p - 1], ph[p - 1], d);
  d = fma(-wx[p], ph[p + 1], d);
  d = fma(-wy[p - P], ph[p - P], d);
  d = fma(-wy[p], ph[p + P], d);
  d = fma(-wz[p - S], ph[p - S], d);
  d = fma(-wz[p], ph[p + S], d);
  return d + rhs[p];
}

// Coarse rhs at (K, J, I): 1/32 of the 12 edge-diagonal red neighbours + 1/8 centre,
// summed in the reference's order (solver_3d.py:649).
template <typename T>
__device__ __forceinline__ T restrict_point3d(const Lvl<T>& f, int K, int J, int I) {
  const int P = f.P;
  const long long S = f.S;
  const long long c = (long long)(2 * K - 1) * S + (long long)(2 * J - 1) * P + (2 * I - 1);
#define JMG_D3(o) defect_point3d(f.phi, f.rhs, f.wx, f.wy, f.wz, f.acc, c + (o), P, S)
  T s = JMG_D3(P + 1);
  s = s + JMG_D3(P - 1);
  s = s + JMG_D3(-P + 1);
  s = s + JMG_D3(-P - 1);
  s = s + JMG_D3(S + 1);
  s = s + JMG_D3(S - 1);
  s = s + JMG_D3(-S + 1);
  s = s + JMG_D3(-S - 1);
  s = s + JMG_D3(S + P);
  s = s + JMG_D3(S - P);
  s = s + JMG_D3(-S + P);
  s = s + JMG_D3(-S - P);
  const T dc = JMG_D3(0);
#undef JMG_D3
  return T(0.03125) * s + T(0.125) * dc;
}

// Prolongated correction at fine interior (k, j, i) (solver_3d.py:667-675). Points with
// exactly two even indices are the bilinear ones, computed only when nu2 <= 0.
template <typename T>
__device__ __forceinline__ bool prolong_point3d(const Lvl<T>& c, int k, int j, int i, bool bilinear,
                                                T* out) {
  const T* pc = c.phi;
  const int P = c.P;
  const long long S = c.S;
  const int ke = !(k & 1), je = !(j & 1), ie = !(i & 1);
  const int ne = ke + je + ie;
  // coarse indices: odd fine f -> (f+1)/2; even fine f -> (f+2)/2 ('+') and f/2 ('-')
  const int kp = ke ? (k + 2) >> 1 : (k + 1) >> 1, km = ke ? (k >> 1) : kp;
  const int jp = je ? (j + 2) >> 1 : (j + 1) >> 1, jm = je ? (j >> 1) : jp;
  const int ip = ie ? (i + 2) >> 1 : (i + 1) >> 1, im = ie ? (i >> 1) : ip;
#define JMG_C3(a, b, d) pc[(long long)(a) * S + (long long)(b) * P + (d)]
  if (ne == 0) {
    *out = JMG_C3(kp, jp, ip);
  } else if (ne == 1) {
    if (ie) *out = T(0.5) * (JMG_C3(kp, jp, ip) + JMG_C3(kp, jp, im));
    else if (je) *out = T(0.5) * (JMG_C3(kp, jp, ip) + JMG_C3(kp, jm, ip));
    else *out = T(0.5) * (JMG_C3(kp, jp, ip) + JMG_C3(km, jp, ip));
  } else if (ne == 2) {
    if (!bilinear) return false;
    if (!ke)  // x and y even
      *out = T(0.25) * (((JMG_C3(kp, jp, ip) + JMG_C3(kp, jm, ip)) + JMG_C3(kp, jp, im)) + JMG_C3(kp, jm, im));
    else if (!je)  // x and z even
      *out = T(0.25) * (((JMG_C3(kp, jp, ip) + JMG_C3(km, jp, ip)) + JMG_C3(kp, jp, im)) + JMG_C3(km, jp, im));
    else  // y and z even
      *out = T(0.25) * (((JMG_C3(kp, jp, ip) + JMG_C3(km, jp, ip)) + JMG_C3(kp, jm, ip)) + JMG_C3(km, jm, ip));
  } else {
    T s = JMG_C3(kp, jp, ip);
    s = s + JMG_C3(km, jp, ip);
    s = s + JMG_C3(kp, jm, ip);
    s = s + JMG_C3(km, jm, ip);
    s = s + JMG_C3(kp, jp, im);
    s = s + JMG_C3(km, jp, im);
    s = s + JMG_C3(kp, jm, im);
    s = s + JMG_C3(km, jm, im);
    *out = T(0.125) * s;
  }
#undef JMG_C3
  return true;
}

// Prolongation by coarse cells, the same values as prolong_point2d / prolong_point3d:
// the fine points (2J-1 .. 2J, 2I-1 .. 2I[, 2K-1 .. 2K]) all interpolate from the coarse
// corners (J .. J+1, I .. I+1[, K .. K+1]); the corners are loaded once and each fine
// value takes its class's formula in the reference's order (solver_2d.py:649-668,
// solver_3d.py:654-677). Neighbouring fine points belong to different classes, so one
// thread per fine point diverges; one per cell does not. Cells run 1 .. m_c per axis.
template <typename T>
__device__ __forceinline__ void prolong_cell2d(const Lvl<T>& f, const Lvl<T>& c, int J, int I, bool diag) {
  const int Pc = c.P;
  const T* pc = c.phi + (long long)J * Pc + I;
  const T c00 = pc[0], c01 = pc[1], c10 = pc[Pc], c11 = pc[Pc + 1];  // c_ab = phi_c(J + a, I + b)
  const int Pf = f.P;
  const int r0 = 2 * J - 1, q0 = 2 * I - 1;  // odd fine row and column of the cell
  T* pf = f.phi + (long long)r0 * Pf + q0;
  const bool rin = r0 >= 2, qin = q0 >= 2;   // the even ones (2J, 2I) are interior
  if (rin && qin) pf[0] = pf[0] + c00;
  if (rin) pf[1] = pf[1] + T(0.5) * (c01 + c00);    // odd row, even column
  if (qin) pf[Pf] = pf[Pf] + T(0.5) * (c10 + c00);  // even row, odd column
  if (diag) pf[Pf + 1] = pf[Pf + 1] + T(0.25) * (((c11 + c01) + c10) + c00);
}

template <typename T>
__device__ __forceinline__ void prolong_cell3d(const Lvl<T>& f, const Lvl<T>& c, int K, int J, int I,
                                               bool bilinear) {
  const long long Sc = c.S;
  const int Pc = c.P;
  const T* pc = c.phi + (long long)K * Sc + (long long)J * Pc + I;
  // corners: cabc = phi_c(K + a, J + b, I + c)
  const T c000 = pc[0], c001 = pc[1], c010 = pc[Pc], c011 = pc[Pc + 1];
  const T c100 = pc[Sc], c101 = pc[Sc + 1], c110 = pc[Sc + Pc], c111 = pc[Sc + Pc + 1];
  const long long Sf = f.S;
  const int Pf = f.P;
  const int k0 = 2 * K - 1, j0 = 2 * J - 1, i0 = 2 * I - 1;  // the odd fine indices of the cell
  T* pf = f.phi + (long long)k0 * Sf + (long long)j0 * Pf + i0;
  const bool kin0 = k0 >= 2, jin0 = j0 >= 2, iin0 = i0 >= 2;  // the even ones are interior
#define JMG_ADD(dk, dj, di, val)              \
  {                                           \
    T* q = pf + (dk) * Sf + (dj) * Pf + (di); \
    *q = *q + (val);                          \
  }
  if (kin0 && jin0 && iin0) JMG_ADD(0, 0, 0, c000);  // (odd, odd, odd): injection
  // one even index: 0.5 (c(kp, jp, ip) + c(.. m ..)), the even axis taking K+1 and K
  if (kin0 && jin0) JMG_ADD(0, 0, 1, T(0.5) * (c001 + c000));
  if (kin0 && iin0) JMG_ADD(0, 1, 0, T(0.5) * (c010 + c000));
  if (jin0 && iin0) JMG_ADD(1, 0, 0, T(0.5) * (c100 + c000));
  if (bilinear) {  // two even indices, computed only when asked
    if (kin0) JMG_ADD(0, 1, 1, T(0.25) * (((c011 + c001) + c010) + c000));
    if (jin0) JMG_ADD(1, 0, 1, T(0.25) * (((c101 + c001) + c100) + c000));
    if (iin0) JMG_ADD(1, 1, 0, T(0.25) * (((c110 + c010) + c100) + c000));
  }
  {  // three even indices: the eight corners in prolong_point3d's order
    T s = c111;
    s = s + c011;
    s = s + c101;
    s = s + c001;
    s = s + c110;
    s = s + c010;
    s = s + c100;
    s = s + c000;
    JMG_ADD(1, 1, 1, T(0.125) * s);
  }
#undef JMG_ADD
}

// Order-preserving bit pattern of |x| for NaN-propagating max reductions: for
// non-negative doubles the IEEE bit pattern is monotone, and a NaN (sign cleared)
// compares above +inf, so the maximum is NaN whenever any difference is NaN. This
// keeps the reference's rule that a NaN distance ends the dynamic loop
// (jnp.max propagates NaN; NaN > epsilon is false).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}

}  // namespace jmg
