// mg_fusedops2d.cuh — the 2D fused operator pairs as per-tile device functions, shared by
// their own grid-wide kernels (mg_fusedops2d.cu) and by the persistent middle-level kernel
// (mg_mid2d.cu), which runs many tiles per block between grid barriers.
//
//   k_smooth_restrict2d   the last pre-smoothing sweep (red then black pass,
//                         solver_2d.py:670-692) followed by the defect and restriction onto
//                         the next level (solver_2d.py:616-647), which also zeroes phi_c
//                         (solver_2d.py:607-608);
//   k_prolong_smooth2d    the prolongation phi += P phi_c (solver_2d.py:612, 649-668)
//                         followed by the first post-smoothing sweep.
//
// A tile recomputes, from the level's arrays, everything its outputs depend on, so no block
// reads what another writes: the smoothed phi goes to the level's second buffer and the
// two buffers swap (twice per visit, so phi ends in the buffer it started in).
//
// Smooth + restrict, per block a CJ x CI tile of coarse points (J0.., I0..). The coarse
// point (J, I) restricts the red-point defects at (2J-1 +- 1, 2I-1 +- 1) and (2J-1, 2I-1),
// the fine footprint rows and columns 2J0-2 .. 2J0+2CJ-2 (likewise for I). A red defect
// reads its point and four black neighbours after the sweep: black values on the
// footprint plus a one-point ring; those read red values on the footprint plus two; those
// read old phi on the footprint plus three. The block owns the fine rows (columns)
// 2J0-1 .. 2J0+2CJ-2 of the smoothed phi.
//
// Prolong + smooth, per block a TJ x TI tile of fine interior points. The black values of
// the tile read red values on the tile plus one; those read the prolongated black values
// (old phi + the class's interpolation) on the tile plus two. Red points are not
// prolongated: the red pass overwrites them without reading them (the reference skips the
// (even, even) points for the same reason when nu2 > 0; its (odd, odd) injections are
// overwritten as well).
//
// Every value is computed with gs_point2d's / defect_point2d's / restrict_point2d's /
// prolong_point2d's arithmetic in the same order, so solves give the same bits as the
// unfused operators (JMG_FUSEDOPS=0 selects those; tests/test_gpu_fused.py compares).

// CG = true reads phi and rhs (arrays that other blocks of the same launch write) through
// L2 only (ld.global.cg), never from a possibly stale L1 line; the coefficient arrays are
// constant during a solve and use ordinary loads. The loaded values are the same either way.
#pragma once
#include "mg_common.cuh"

namespace jmg {

template <bool CG, typename T>
__device__ __forceinline__ T ldx(const T* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}


// ---- smooth + restrict ----------------------------------------------------------------

template <typename T, int CJ, int CI>
struct SR {
  static constexpr int DR = 2 * CJ + 1, DC = 2 * CI + 1;  // footprint (red defects)
  static constexpr int NR = DR + 4, NC = DC + 4;          // new phi: footprint + 2
  static constexpr int OR = DR + 6, OC = DC + 6;          // old phi: footprint + 3
  static constexpr size_t smem = sizeof(T) * ((size_t)OR * OC + (size_t)NR * NC + (size_t)DR * DC);
};

template <typename T, int CJ, int CI, int NT, bool CG>
__device__ __forceinline__ void smooth_restrict_tile(const Lvl<T>& f, T* __restrict__ out, const Lvl<T>& c,
                                                     int zero_in, int by, int bx, unsigned char* smraw) {
  using G = SR<T, CJ, CI>;
  T* Old = reinterpret_cast<T*>(smraw);  // [OR][OC], fine (fr0 - 3 + r, fc0 - 3 + q)
  T* New = Old + G::OR * G::OC;          // [NR][NC], fine (fr0 - 2 + r, fc0 - 2 + q)
  T* Def = New + G::NR * G::NC;          // [DR][DC], fine (fr0 + r, fc0 + q)
  const int J0 = by * CJ, I0 = bx * CI;
  const int fr0 = 2 * J0 - 2, fc0 = 2 * I0 - 2;
  const int tid = threadIdx.x;
  const long long P = f.P;
  const int mx = f.mx, my = f.my;
  // 1. old phi (zero outside the padded array; not read from a zero initial guess)
  if (!zero_in) {
    constexpr int N = G::OR * G::OC, U = (N + NT - 1) / NT;
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      v[u] = T(0);
      if (t < N) {
        const int r = t / G::OC, q = t - r * G::OC;
        const int i = fr0 - 3 + r, j = fc0 - 3 + q;
        if (i >= 0 && j >= 0 && i <= my + 2 && j <= mx + 2) v[u] = ldx<CG>(f.phi + i * P + j);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      if (t < N) Old[t] = v[u];
    }
  }
  __syncthreads();
  // 2. red pass on the footprint + 2 (i + j even); non-interior points stay zero
  {
    constexpr int XR = (G::NC + 1) / 2, N = G::NR * XR, U = (N + NT - 1) / NT;
    T cwxm[U], cwxp[U], cwym[U], cwyp[U], crh[U], cinv[U];
    int slot[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      slot[u] = -1;
      if (t < N) {
        const int r = t / XR, xp = t - r * XR;
        const int i = fr0 - 2 + r;
        const int q = 2 * xp + ((i + fc0 - 2) & 1);  // j = fc0 - 2 + q with i + j even
        const int j = fc0 - 2 + q;
        if (q < G::NC) {
          slot[u] = r * G::NC + q;
          if (i >= 2 && i <= my && j >= 2 && j <= mx) {
            const long long p = i * P + j;
            crh[u] = ldx<CG>(f.rhs + p);
            cinv[u] = f.invd[p];
            if (!zero_in) {
              cwxm[u] = f.wx[p - 1];
              cwxp[u] = f.wx[p];
              cwym[u] = f.wy[p - P];
              cwyp[u] = f.wy[p];
            }
          } else {
            slot[u] = -2 - slot[u];  // exterior: value 0
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (slot[u] == -1) continue;
      if (slot[u] < -1) {
        New[-2 - slot[u]] = T(0);
        continue;
      }
      const int r = slot[u] / G::NC, q = slot[u] - r * G::NC;
      T v;
      if (zero_in) {
        v = (T(0) - crh[u]) * cinv[u];
      } else {
        const T* o = Old + (r + 1) * G::OC + (q + 1);  // the same fine point in Old
        T s = cwyp[u] * o[G::OC];
        s = fma(cwym[u], o[-G::OC], s);
        s = fma(cwxp[u], o[1], s);
        s = fma(cwxm[u], o[-1], s);
        s = s - crh[u];
        v = s * cinv[u];
      }
      New[slot[u]] = v;
    }
  }
  __syncthreads();
  // 3. black pass on the footprint + 1 (i + j odd) from the new red values
  {
    constexpr int BR = G::DR + 2, BC = G::DC + 2;  // footprint + 1
    constexpr int XB = (BC + 1) / 2, N = BR * XB, U = (N + NT - 1) / NT;
    T cwxm[U], cwxp[U], cwym[U], cwyp[U], crh[U], cinv[U];
    int slot[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      slot[u] = -1;
      if (t < N) {
        const int r = t / XB, xp = t - r * XB;
        const int i = fr0 - 1 + r;
        const int q = 2 * xp + ((i + fc0 - 1 + 1) & 1);  // j = fc0 - 1 + q with i + j odd
        const int j = fc0 - 1 + q;
        if (q < BC) {
          slot[u] = (r + 1) * G::NC + (q + 1);  // position in New
          if (i >= 2 && i <= my && j >= 2 && j <= mx) {
            const long long p = i * P + j;
            crh[u] = ldx<CG>(f.rhs + p);
            cinv[u] = f.invd[p];
            cwxm[u] = f.wx[p - 1];
            cwxp[u] = f.wx[p];
            cwym[u] = f.wy[p - P];
            cwyp[u] = f.wy[p];
          } else {
            slot[u] = -2 - slot[u];
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (slot[u] == -1) continue;
      if (slot[u] < -1) {
        New[-2 - slot[u]] = T(0);
        continue;
      }
      const T* n = New + slot[u];
      T s = cwyp[u] * n[G::NC];
      s = fma(cwym[u], n[-G::NC], s);
      s = fma(cwxp[u], n[1], s);
      s = fma(cwxm[u], n[-1], s);
      s = s - crh[u];
      New[slot[u]] = s * cinv[u];
    }
  }
  __syncthreads();
  // 4. red defects on the footprint (0 outside the interior); the owned smoothed phi out
  {
    constexpr int XR = (G::DC + 1) / 2, N = G::DR * XR, U = (N + NT - 1) / NT;
    T cac[U], cwxm[U], cwxp[U], cwym[U], cwyp[U], crh[U];
    int slot[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      slot[u] = -1;
      if (t < N) {
        const int r = t / XR, xp = t - r * XR;
        const int i = fr0 + r;
        const int q = 2 * xp + ((i + fc0) & 1);
        const int j = fc0 + q;
        if (q < G::DC) {
          slot[u] = r * G::DC + q;
          if (i >= 2 && i <= my && j >= 2 && j <= mx) {
            const long long p = i * P + j;
            cac[u] = f.acc[p];
            cwxm[u] = f.wx[p - 1];
            cwxp[u] = f.wx[p];
            cwym[u] = f.wy[p - P];
            cwyp[u] = f.wy[p];
            crh[u] = ldx<CG>(f.rhs + p);
          } else {
            slot[u] = -2 - slot[u];
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (slot[u] == -1) continue;
      if (slot[u] < -1) {
        Def[-2 - slot[u]] = T(0);
        continue;
      }
      const int r = slot[u] / G::DC, q = slot[u] - r * G::DC;
      const T* n = New + (r + 2) * G::NC + (q + 2);
      // defect_point2d's order
      T d = cac[u] * n[0];
      d = fma(-cwxm[u], n[-1], d);
      d = fma(-cwxp[u], n[1], d);
      d = fma(-cwym[u], n[-G::NC], d);
      d = fma(-cwyp[u], n[G::NC], d);
      d = d + crh[u];
      Def[slot[u]] = d;
    }
    // owned fine points: rows fr0 + 1 .. fr0 + 2CJ, columns fc0 + 1 .. fc0 + 2CI (interior)
    constexpr int OWN = (2 * CJ) * (2 * CI);
    for (int t = tid; t < OWN; t += NT) {
      const int r = t / (2 * CI), q = t - r * (2 * CI);
      const int i = fr0 + 1 + r, j = fc0 + 1 + q;
      if (i >= 2 && i <= my && j >= 2 && j <= mx) out[i * P + j] = New[(r + 3) * G::NC + (q + 3)];
    }
  }
  __syncthreads();
  // 5. coarse rhs (restrict_point2d's order) and phi_c = 0 over the padded coarse tile
  const long long Pc = c.P;
  for (int t = tid; t < CJ * CI; t += NT) {
    const int J = J0 + t / CI, I = I0 + t % CI;
    if (J > c.my + 2 || I > c.mx + 2) continue;
    T v = T(0);
    if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) {
      const int r = 2 * J - 1 - fr0, q = 2 * I - 1 - fc0;
      const T* d = Def + r * G::DC + q;
      const T s = ((d[G::DC + 1] + d[G::DC - 1]) + d[-G::DC + 1]) + d[-G::DC - 1];
      v = T(0.0625) * s + T(0.25) * d[0];
    }
    c.rhs[J * Pc + I] = v;
    c.phi[J * Pc + I] = T(0);
  }
}

// ---- prolong + smooth -------------------------------------------------------------------

template <typename T, int TJ, int TI>
struct PS {
  static constexpr int BR = TJ + 4, BC = TI + 4;  // prolongated black values: tile + 2
  static constexpr int RR = TJ + 2, RC = TI + 2;  // new red values: tile + 1
  static constexpr size_t smem = sizeof(T) * ((size_t)BR * BC + (size_t)RR * RC);
};

template <typename T, int TJ, int TI, int NT, bool CG>
__device__ __forceinline__ void prolong_smooth_tile(const Lvl<T>& f, T* __restrict__ out, const Lvl<T>& c, int by,
                                                    int bx, unsigned char* smraw) {
  using G = PS<T, TJ, TI>;
  T* Blk = reinterpret_cast<T*>(smraw);  // [BR][BC], fine (i0 - 2 + r, j0 - 2 + q)
  T* Red = Blk + G::BR * G::BC;          // [RR][RC], fine (i0 - 1 + r, j0 - 1 + q)
  const int i0 = 2 + by * TJ, j0 = 2 + bx * TI;
  const int tid = threadIdx.x;
  const long long P = f.P, Pc = c.P;
  const int mx = f.mx, my = f.my;
  // 1. black points of the tile + 2: old phi + the interpolated correction
  {
    constexpr int XB = (G::BC + 1) / 2, N = G::BR * XB, U = (N + NT - 1) / NT;
    T old[U], ca[U], cb[U];
    int slot[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      slot[u] = -1;
      if (t < N) {
        const int r = t / XB, xp = t - r * XB;
        const int i = i0 - 2 + r;
        const int q = 2 * xp + ((i + j0 - 2 + 1) & 1);  // j = j0 - 2 + q with i + j odd
        const int j = j0 - 2 + q;
        if (q < G::BC) {
          slot[u] = r * G::BC + q;
          if (i >= 2 && i <= my && j >= 2 && j <= mx) {
            old[u] = ldx<CG>(f.phi + i * P + j);
            if (i & 1) {  // odd row, even column: linear in x (prolong_point2d)
              const long long rc = (long long)((i + 1) >> 1) * Pc;
              ca[u] = ldx<CG>(c.phi + rc + ((j + 2) >> 1));
              cb[u] = ldx<CG>(c.phi + rc + (j >> 1));
            } else {      // even row, odd column: linear in y
              const int cj = (j + 1) >> 1;
              ca[u] = ldx<CG>(c.phi + (long long)((i + 2) >> 1) * Pc + cj);
              cb[u] = ldx<CG>(c.phi + (long long)(i >> 1) * Pc + cj);
            }
          } else {
            slot[u] = -2 - slot[u];
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (slot[u] == -1) continue;
      if (slot[u] < -1) {
        Blk[-2 - slot[u]] = T(0);
        continue;
      }
      Blk[slot[u]] = old[u] + T(0.5) * (ca[u] + cb[u]);
    }
  }
  __syncthreads();
  // 2. red pass on the tile + 1
  {
    constexpr int XR = (G::RC + 1) / 2, N = G::RR * XR, U = (N + NT - 1) / NT;
    T cwxm[U], cwxp[U], cwym[U], cwyp[U], crh[U], cinv[U];
    int slot[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      slot[u] = -1;
      if (t < N) {
        const int r = t / XR, xp = t - r * XR;
        const int i = i0 - 1 + r;
        const int q = 2 * xp + ((i + j0 - 1) & 1);  // i + j even
        const int j = j0 - 1 + q;
        if (q < G::RC) {
          slot[u] = r * G::RC + q;
          if (i >= 2 && i <= my && j >= 2 && j <= mx) {
            const long long p = i * P + j;
            crh[u] = ldx<CG>(f.rhs + p);
            cinv[u] = f.invd[p];
            cwxm[u] = f.wx[p - 1];
            cwxp[u] = f.wx[p];
            cwym[u] = f.wy[p - P];
            cwyp[u] = f.wy[p];
          } else {
            slot[u] = -2 - slot[u];
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (slot[u] == -1) continue;
      if (slot[u] < -1) {
        Red[-2 - slot[u]] = T(0);
        continue;
      }
      const int r = slot[u] / G::RC, q = slot[u] - r * G::RC;
      const T* b = Blk + (r + 1) * G::BC + (q + 1);
      T s = cwyp[u] * b[G::BC];
      s = fma(cwym[u], b[-G::BC], s);
      s = fma(cwxp[u], b[1], s);
      s = fma(cwxm[u], b[-1], s);
      s = s - crh[u];
      Red[slot[u]] = s * cinv[u];
    }
  }
  __syncthreads();
  // 3. black pass on the tile; both colours of the tile out
  {
    constexpr int XB = TI / 2, N = TJ * XB, U = (N + NT - 1) / NT;
    T cwxm[U], cwxp[U], cwym[U], cwyp[U], crh[U], cinv[U];
    int ok[U];
    long long pp[U];
    int rr[U], qq[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = tid + u * NT;
      ok[u] = 0;
      if (t < N) {
        const int r = t / XB, xp = t - r * XB;
        const int i = i0 + r;
        const int q = 2 * xp + ((i + j0 + 1) & 1);  // i + j odd
        const int j = j0 + q;
        rr[u] = r;
        qq[u] = q;
        if (i <= my && j <= mx) {
          const long long p = i * P + j;
          ok[u] = 1;
          pp[u] = p;
          crh[u] = ldx<CG>(f.rhs + p);
          cinv[u] = f.invd[p];
          cwxm[u] = f.wx[p - 1];
          cwxp[u] = f.wx[p];
          cwym[u] = f.wy[p - P];
          cwyp[u] = f.wy[p];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (!ok[u]) continue;
      const T* n = Red + (rr[u] + 1) * G::RC + (qq[u] + 1);
      T s = cwyp[u] * n[G::RC];
      s = fma(cwym[u], n[-G::RC], s);
      s = fma(cwxp[u], n[1], s);
      s = fma(cwxm[u], n[-1], s);
      s = s - crh[u];
      out[pp[u]] = s * cinv[u];
    }
    for (int t = tid; t < TJ * (TI / 2); t += NT) {
      const int r = t / (TI / 2), xp = t - r * (TI / 2);
      const int i = i0 + r;
      const int q = 2 * xp + ((i + j0) & 1);  // i + j even
      const int j = j0 + q;
      if (i <= my && j <= mx) out[i * P + j] = Red[(r + 1) * G::RC + (q + 1)];
    }
  }
}

// tile shapes: FP32 16 x 32 coarse points (512 threads, 30 KB) for smooth + restrict and
// 32 x 64 fine points (512 threads, 19 KB) for prolong + smooth; FP64 8 x 32 (256
// threads, 33 KB) and 16 x 64 (256 threads, 20 KB)
template <typename T>
struct FusedShape;
template <>
struct FusedShape<float> {
  static constexpr int CJ = 16, CI = 32, NT_SR = 512, TJ = 32, TI = 64, NT_PS = 512;
};
template <>
struct FusedShape<double> {
  static constexpr int CJ = 8, CI = 32, NT_SR = 256, TJ = 16, TI = 64, NT_PS = 256;
};

}  // namespace jmg
