// mg_coarse.cu — the coarse levels of a cycle on one thread-block cluster.
//
// Below ~20 000 points per level a grid-wide launch per operator costs more in launch
// latency than in work, but one SM is too slow for the work itself: GB300 issues about
// two FP64 FMAs per clock per SM, so a 64^2 level alone keeps a single block busy for
// tens of microseconds per cycle. k_coarse_cluster runs the reference's recursion
// (solver_2d.py:582-614, solver_3d.py:587-619) for every level from `lev0` down to L-2
// on a cluster of R CTAs (16 where the GPU allows it, else 8), one CTA per SM:
//   * every level's rows (2D: j; 3D: the (k, j) rows) are split into R contiguous
//     blocks, one per CTA; a CTA keeps phi, rhs and the coefficient arrays (wx, wy, wz,
//     acc, invd) of its rows in its own shared memory, loaded from global memory at
//     entry; levels of at most kLocalPoints points live whole in CTA 0;
//   * a point's neighbours in other CTAs' rows are read through distributed shared
//     memory (generic pointers from cluster.map_shared_rank);
//   * passes that touch a spread level end with a cluster barrier (release/acquire),
//     passes on CTA-0-only levels with a block barrier;
//   * at exit every CTA writes phi of its rows of `lev0` back to global memory.
// The arithmetic of every point is that of the grid-wide kernels (mg_common.cuh), in
// the reference's order, so results are bit-identical to them.
#include <cooperative_groups.h>

#include <type_traits>

#include "mg_common.cuh"
#include "mg_kernels.h"

namespace cg = cooperative_groups;

namespace jmg {

namespace {

constexpr int kThreads = 512;
constexpr int kLocalPoints = 1024;  // levels up to this many padded points live in CTA 0

// array slots of a level block
enum { A_PHI = 0, A_RHS, A_WX, A_WY, A_ACC, A_INVD, A_WZ };

template <typename T>
struct Ctx {
  T* sm;                 // this CTA's shared memory
  T* const* rb;          // generic pointers to every CTA's shared memory (rank-indexed)
  int me;
};

// one level as seen from one CTA. Row s of array a of the level sits in the CTA that
// owns s at element off + (a * rpr + ls) * rp, ls = s - first row of that CTA.
template <typename T, int DIM>
struct DLevel {
  int off, nx, ny, rp, nrows, rpr, dist, as;
  int mx, my, mz;
  int s0, s1;  // rows owned by this CTA ([0, 0) for none)

  __device__ void init(const ClusterLevel& L, int me) {
    off = L.off;
    nx = L.nx;
    ny = L.ny;
    rp = L.rp;
    nrows = L.nrows;
    rpr = L.rpr;
    dist = L.dist;
    as = rpr * rp;
    mx = L.m[0];
    my = L.m[1];
    mz = L.m[2];
    if (dist) {
      s0 = min(nrows, me * rpr);
      s1 = min(nrows, s0 + rpr);
    } else {
      s0 = 0;
      s1 = me == 0 ? nrows : 0;
    }
  }
  // array-0 (phi) pointer of row s, wherever it lives; array a is at + a * as
  __device__ __forceinline__ T* rowp(const Ctx<T>& c, int s) const {
    if (!dist) return (c.me == 0 ? c.sm : c.rb[0]) + off + s * rp;  // the level lives in CTA 0
    if (s >= s0 && s < s0 + rpr) return c.sm + off + (s - s0) * rp;
    const int r = s / rpr;
    return c.rb[r] + off + (s - r * rpr) * rp;
  }
  // owned row (local)
  __device__ __forceinline__ T* own(const Ctx<T>& c, int s) const { return c.sm + off + (s - s0) * rp; }
};

// ---- point arithmetic on distributed rows (same order as mg_common.cuh) -----------------
// q: the point's row, qn / qs: rows j+1 / j-1, qu / qd: rows k+1 / k-1 (3D); arrays at
// multiples of `as`.

template <typename T, int DIM>
__device__ __forceinline__ T d_gs(const T* q, const T* qn, const T* qs, const T* qu, const T* qd, int as, int i) {
  T s;
  if (DIM == 3) {
    s = q[A_WZ * as + i] * qu[i];
    s = fma(qd[A_WZ * as + i], qd[i], s);
    s = fma(q[A_WY * as + i], qn[i], s);
  } else {
    s = q[A_WY * as + i] * qn[i];
  }
  s = fma(qs[A_WY * as + i], qs[i], s);
  s = fma(q[A_WX * as + i], q[i + 1], s);
  s = fma(q[A_WX * as + i - 1], q[i - 1], s);
  s = s - q[A_RHS * as + i];
  return s * q[A_INVD * as + i];
}

template <typename T, int DIM>
__device__ __forceinline__ T d_defect(const T* q, const T* qn, const T* qs, const T* qu, const T* qd, int as, int i) {
  T d = q[A_ACC * as + i] * q[i];
  d = fma(-q[A_WX * as + i - 1], q[i - 1], d);
  d = fma(-q[A_WX * as + i], q[i + 1], d);
  d = fma(-qs[A_WY * as + i], qs[i], d);
  d = fma(-q[A_WY * as + i], qn[i], d);
  if (DIM == 3) {
    d = fma(-qd[A_WZ * as + i], qd[i], d);
    d = fma(-q[A_WZ * as + i], qu[i], d);
  }
  return d + q[A_RHS * as + i];
}

// defect at fine (k, j, i), looking its rows up
template <typename T, int DIM>
__device__ __forceinline__ T d_defect_at(const Ctx<T>& c, const DLevel<T, DIM>& f, int k, int j, int i) {
  const int s = k * f.ny + j;
  const T* q = f.rowp(c, s);
  const T* qn = f.rowp(c, s + 1);
  const T* qs = f.rowp(c, s - 1);
  const T* qu = DIM == 3 ? f.rowp(c, s + f.ny) : nullptr;
  const T* qd = DIM == 3 ? f.rowp(c, s - f.ny) : nullptr;
  return d_defect<T, DIM>(q, qn, qs, qu, qd, f.as, i);
}

template <typename T, int DIM>
__device__ __forceinline__ T d_restrict(const Ctx<T>& c, const DLevel<T, DIM>& f, int K, int J, int I) {
  const int i = 2 * I - 1, j = 2 * J - 1;
  if constexpr (DIM == 2) {
    // fine rows j-2 .. j+2
    const T* r0 = f.rowp(c, j - 2);
    const T* r1 = f.rowp(c, j - 1);
    const T* r2 = f.rowp(c, j);
    const T* r3 = f.rowp(c, j + 1);
    const T* r4 = f.rowp(c, j + 2);
    const int as = f.as;
    const T dne = d_defect<T, 2>(r3, r4, r2, nullptr, nullptr, as, i + 1);
    const T dnw = d_defect<T, 2>(r3, r4, r2, nullptr, nullptr, as, i - 1);
    const T dse = d_defect<T, 2>(r1, r2, r0, nullptr, nullptr, as, i + 1);
    const T dsw = d_defect<T, 2>(r1, r2, r0, nullptr, nullptr, as, i - 1);
    const T dc = d_defect<T, 2>(r2, r3, r1, nullptr, nullptr, as, i);
    return T(0.0625) * (((dne + dnw) + dse) + dsw) + T(0.25) * dc;
  } else {
    const int k = 2 * K - 1;
    T s = d_defect_at<T, 3>(c, f, k, j + 1, i + 1);
    s = s + d_defect_at<T, 3>(c, f, k, j + 1, i - 1);
    s = s + d_defect_at<T, 3>(c, f, k, j - 1, i + 1);
    s = s + d_defect_at<T, 3>(c, f, k, j - 1, i - 1);
    s = s + d_defect_at<T, 3>(c, f, k + 1, j, i + 1);
    s = s + d_defect_at<T, 3>(c, f, k + 1, j, i - 1);
    s = s + d_defect_at<T, 3>(c, f, k - 1, j, i + 1);
    s = s + d_defect_at<T, 3>(c, f, k - 1, j, i - 1);
    s = s + d_defect_at<T, 3>(c, f, k + 1, j + 1, i);
    s = s + d_defect_at<T, 3>(c, f, k + 1, j - 1, i);
    s = s + d_defect_at<T, 3>(c, f, k - 1, j + 1, i);
    s = s + d_defect_at<T, 3>(c, f, k - 1, j - 1, i);
    return T(0.03125) * s + T(0.125) * d_defect_at<T, 3>(c, f, k, j, i);
  }
}

// prolongated correction at fine (k, j, i) from the coarse level (prolong_point2d/3d)
template <typename T, int DIM>
__device__ __forceinline__ bool d_prolong(const Ctx<T>& c, const DLevel<T, DIM>& cv, int k, int j, int i,
                                          bool diag, T* out) {
  if constexpr (DIM == 2) {
    const bool jo = j & 1, io = i & 1;
    if (jo && io) {
      *out = cv.rowp(c, (j + 1) >> 1)[(i + 1) >> 1];
    } else if (jo) {
      const T* r = cv.rowp(c, (j + 1) >> 1);
      *out = T(0.5) * (r[(i + 2) >> 1] + r[i >> 1]);
    } else if (io) {
      const int ci = (i + 1) >> 1;
      *out = T(0.5) * (cv.rowp(c, (j + 2) >> 1)[ci] + cv.rowp(c, j >> 1)[ci]);
    } else {
      if (!diag) return false;
      const T* rp = cv.rowp(c, (j + 2) >> 1);
      const T* rm = cv.rowp(c, j >> 1);
      const int cp = (i + 2) >> 1, cm = i >> 1;
      *out = T(0.25) * (((rp[cp] + rm[cp]) + rp[cm]) + rm[cm]);
    }
    return true;
  } else {
    auto C = [&](int K, int J, int I) -> T { return cv.rowp(c, K * cv.ny + J)[I]; };
    const int ke = !(k & 1), je = !(j & 1), ie = !(i & 1);
    const int ne = ke + je + ie;
    const int kp = ke ? (k + 2) >> 1 : (k + 1) >> 1, km = ke ? (k >> 1) : kp;
    const int jp = je ? (j + 2) >> 1 : (j + 1) >> 1, jm = je ? (j >> 1) : jp;
    const int ip = ie ? (i + 2) >> 1 : (i + 1) >> 1, im = ie ? (i >> 1) : ip;
    if (ne == 0) {
      *out = C(kp, jp, ip);
    } else if (ne == 1) {
      if (ie) *out = T(0.5) * (C(kp, jp, ip) + C(kp, jp, im));
      else if (je) *out = T(0.5) * (C(kp, jp, ip) + C(kp, jm, ip));
      else *out = T(0.5) * (C(kp, jp, ip) + C(km, jp, ip));
    } else if (ne == 2) {
      if (!diag) return false;
      if (!ke) *out = T(0.25) * (((C(kp, jp, ip) + C(kp, jm, ip)) + C(kp, jp, im)) + C(kp, jm, im));
      else if (!je) *out = T(0.25) * (((C(kp, jp, ip) + C(km, jp, ip)) + C(kp, jp, im)) + C(km, jp, im));
      else *out = T(0.25) * (((C(kp, jp, ip) + C(km, jp, ip)) + C(kp, jm, ip)) + C(km, jm, ip));
    } else {
      T s = C(kp, jp, ip);
      s = s + C(km, jp, ip);
      s = s + C(kp, jm, ip);
      s = s + C(km, jm, ip);
      s = s + C(kp, jp, im);
      s = s + C(km, jp, im);
      s = s + C(kp, jm, im);
      s = s + C(km, jm, im);
      *out = T(0.125) * s;
    }
    return true;
  }
}

// ---- passes ------------------------------------------------------------------------------

template <typename T, int DIM>
__device__ __forceinline__ bool interior_row(const DLevel<T, DIM>& v, int s, int* k, int* j) {
  *k = DIM == 3 ? s / v.ny : 0;
  *j = DIM == 3 ? s - *k * v.ny : s;
  return *j >= 2 && *j <= v.my && (DIM == 2 || (*k >= 2 && *k <= v.mz));
}

template <typename T, int DIM>
__device__ void p_sweep_colour(const Ctx<T>& c, const DLevel<T, DIM>& v, int colour) {
  const int par = DIM == 2 ? colour : (first_color_parity<3>() + colour) & 1;
  const int hx = v.mx / 2;
  const int n = (v.s1 - v.s0) * hx;
  for (int t = threadIdx.x; t < n; t += kThreads) {
    const int q = t / hx;
    const int s = v.s0 + q;
    int k, j;
    if (!interior_row(v, s, &k, &j)) continue;
    const int i = 2 + ((j + k + par) & 1) + 2 * (t - q * hx);
    if (i > v.mx) continue;
    T* r = v.own(c, s);
    const T* rn = v.rowp(c, s + 1);
    const T* rs = v.rowp(c, s - 1);
    const T* ru = DIM == 3 ? v.rowp(c, s + v.ny) : nullptr;
    const T* rd = DIM == 3 ? v.rowp(c, s - v.ny) : nullptr;
    r[i] = d_gs<T, DIM>(r, rn, rs, ru, rd, v.as, i);
  }
}

template <typename T, int DIM>
__device__ void p_restrict(const Ctx<T>& c, const DLevel<T, DIM>& f, const DLevel<T, DIM>& cv) {
  const int n = (cv.s1 - cv.s0) * cv.nx;
  for (int t = threadIdx.x; t < n; t += kThreads) {
    const int q = t / cv.nx, I = t - q * cv.nx;
    const int s = cv.s0 + q;
    int K, J;
    T val = T(0);
    if (interior_row(cv, s, &K, &J) && I >= 2 && I <= cv.mx) val = d_restrict<T, DIM>(c, f, K, J, I);
    T* r = cv.own(c, s);
    r[A_RHS * cv.as + I] = val;
    r[I] = T(0);
  }
}

template <typename T, int DIM>
__device__ void p_prolong(const Ctx<T>& c, const DLevel<T, DIM>& f, const DLevel<T, DIM>& cv, bool diag) {
  const int nx = f.mx - 1;
  const int n = (f.s1 - f.s0) * nx;
  for (int t = threadIdx.x; t < n; t += kThreads) {
    const int q = t / nx, i = 2 + (t - q * nx);
    int k, j;
    if (!interior_row(f, f.s0 + q, &k, &j)) continue;
    T val;
    if (d_prolong<T, DIM>(c, cv, k, j, i, diag, &val)) {
      T* ph = f.own(c, f.s0 + q);
      ph[i] = ph[i] + val;
    }
  }
}


template <typename T, int DIM>
__global__ void __launch_bounds__(kThreads) k_coarse_cluster(const LvlTable<T>* __restrict__ tab, ClusterLayout lay,
                                                             CycleParams cp, int fcycle0, int skip_pre0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T* rb[kMaxClusterRanks];
  cg::cluster_group cluster = cg::this_cluster();
  Ctx<T> c;
  c.sm = reinterpret_cast<T*>(smem_raw);
  c.rb = rb;
  c.me = (int)cluster.block_rank();
  if (threadIdx.x < lay.ranks) rb[threadIdx.x] = cluster.map_shared_rank(c.sm, (int)threadIdx.x);
  const int lev0 = lay.lev0;

  // stage the owned rows in shared memory: the coefficients of every level, phi and rhs
  // of the entry level, in 16-byte loads through L2, four in flight per thread. A global
  // row starts on a 64-byte boundary and its pitch covers the copied rp >= nx elements.
  using V = typename std::conditional<sizeof(T) == 8, double2, float4>::type;
  constexpr int kV = 16 / sizeof(T);  // elements per load
  for (int l = lev0; l <= lay.last; ++l) {
    DLevel<T, DIM> v;
    v.init(lay.l[l - lev0], c.me);
    const Lvl<T>& g = tab->l[l];
    const int cpr = v.rp / kV;  // loads per row
    const int n = (v.s1 - v.s0) * cpr;
    const int na = DIM == 3 ? 7 : 6;
    for (int a = l == lev0 ? A_PHI : A_WX; a < na; ++a) {
      const T* src = a == A_PHI ? g.phi : a == A_RHS ? g.rhs : a == A_WX ? g.wx : a == A_WY ? g.wy
                   : a == A_ACC ? g.acc : a == A_INVD ? g.invd : g.wz;
      T* dst = c.sm + v.off + a * v.as;
      for (int t0 = threadIdx.x; t0 < n; t0 += 4 * kThreads) {
        V buf[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * kThreads;
          if (t < n) {
            const int q = t / cpr, e = (t - q * cpr) * kV;
            const int s = v.s0 + q;
            const int k = DIM == 3 ? s / v.ny : 0, j = s - k * v.ny;
            buf[u] = __ldcg(reinterpret_cast<const V*>(src + (long long)k * g.S + (long long)j * g.P + e));
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * kThreads;
          if (t < n) {
            const int q = t / cpr, e = (t - q * cpr) * kV;
            *reinterpret_cast<V*>(dst + q * v.rp + e) = buf[u];
          }
        }
      }
    }
  }
  cluster.sync();

  // pass bookkeeping: a pass on a spread level, or one following a CTA-0-only pass that
  // the next pass reads remotely, is fenced by cluster barriers
  bool prev_local = false;
  auto begin = [&](bool spread) {
    if (spread && prev_local) cluster.sync();
  };
  auto end = [&](bool spread) {
    if (spread) cluster.sync();
    else __syncthreads();
    prev_local = !spread;
  };
  auto sweep = [&](const DLevel<T, DIM>& v) {
    for (int colour = 0; colour < 2; ++colour) {
      begin(v.dist);
      if (v.s1 > v.s0) p_sweep_colour<T, DIM>(c, v, colour);
      end(v.dist);
    }
  };

  struct Frame {
    int lev, stage, g;
    bool fcycle, skip_pre;
  };
  Frame st[kMaxLevels + 1];
  int sp = 0;
  st[sp++] = Frame{lev0, 0, 0, fcycle0 != 0, skip_pre0 != 0};
  while (sp > 0) {
    Frame& fr = st[sp - 1];
    DLevel<T, DIM> vf;
    vf.init(lay.l[fr.lev - lev0], c.me);
    if (fr.lev == cp.last_level) {
      for (int s = 0; s < cp.nu1 + cp.nu2; ++s) sweep(vf);
      --sp;
      continue;
    }
    DLevel<T, DIM> vc;
    vc.init(lay.l[fr.lev + 1 - lev0], c.me);
    const bool spread = vf.dist || vc.dist;
    if (fr.stage == 0) {
      if (!fr.skip_pre)
        for (int s = 0; s < cp.nu1; ++s) sweep(vf);
      begin(spread);
      if (vc.s1 > vc.s0) p_restrict<T, DIM>(c, vf, vc);
      end(spread);
      fr.stage = fr.fcycle ? 1 : 2;
      fr.g = 0;
    }
    if (fr.stage == 1) {
      if (fr.g < cp.gamma) {
        ++fr.g;
        st[sp++] = Frame{fr.lev + 1, 0, 0, true, false};
        continue;
      }
      fr.stage = 2;
      fr.g = 0;
    }
    if (fr.stage == 2) {
      if (fr.g < cp.gamma) {
        ++fr.g;
        st[sp++] = Frame{fr.lev + 1, 0, 0, false, false};
        continue;
      }
      fr.stage = 3;
    }
    begin(spread);
    if (vf.s1 > vf.s0) p_prolong<T, DIM>(c, vf, vc, cp.diag != 0);
    end(spread);
    for (int s = 0; s < cp.nu2; ++s) sweep(vf);
    --sp;
  }

  // write phi of the owned rows of the entry level back
  {
    DLevel<T, DIM> v;
    v.init(lay.l[0], c.me);
    const Lvl<T>& g = tab->l[lev0];
    const int n = (v.s1 - v.s0) * v.nx;
    for (int t = threadIdx.x; t < n; t += kThreads) {
      const int q = t / v.nx, i = t - q * v.nx;
      const int s = v.s0 + q;
      const int k = DIM == 3 ? s / v.ny : 0, j = s - k * v.ny;
      g.phi[(long long)k * g.S + (long long)j * g.P + i] = c.sm[v.off + q * v.rp + i];
    }
  }
  // no CTA leaves while another may still read its shared memory
  cluster.sync();
}

}  // namespace

int cluster_layout(int dim, const int m[][3], int lev0, int last, int ranks, ClusterLayout* out) {
  if (last - lev0 + 1 > kMaxLevels || ranks > kMaxClusterRanks || ranks < 1) return 1;
  ClusterLayout& lay = *out;
  lay.lev0 = lev0;
  lay.last = last;
  lay.ranks = ranks;
  const int na = dim == 3 ? 7 : 6;
  long long off = 0;
  for (int l = lev0; l <= last; ++l) {
    ClusterLevel& L = lay.l[l - lev0];
    L.m[0] = m[l][0];
    L.m[1] = m[l][1];
    L.m[2] = dim == 3 ? m[l][2] : 0;
    L.nx = m[l][0] + 3;
    L.ny = m[l][1] + 3;
    L.rp = (L.nx + 3) & ~3;  // row pitch: 16-byte rows for either element size
    const int nz = dim == 3 ? m[l][2] + 3 : 1;
    L.nrows = L.ny * nz;
    L.dist = (long long)L.nx * L.nrows > kLocalPoints && ranks > 1;
    L.rpr = L.dist ? (L.nrows + ranks - 1) / ranks : L.nrows;
    L.off = (int)off;
    off += (long long)na * L.rpr * L.rp;
  }
  lay.elems = off;
  return 0;
}

template <typename T>
int prepare_coarse_cluster(int dim, size_t smem_bytes, int ranks) {
  const void* fn = dim == 2 ? (const void*)k_coarse_cluster<T, 2> : (const void*)k_coarse_cluster<T, 3>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes) != cudaSuccess) return 1;
  if (ranks > 8 && cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
    return 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ranks);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem_bytes;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ranks;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return nclusters >= 1 ? 0 : 1;
}

template <typename T>
void launch_coarse_cluster(int dim, const LvlTable<T>* tab, const ClusterLayout& lay, const CycleParams& cp,
                           int fcycle, int skip_pre, size_t smem_bytes, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(lay.ranks);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem_bytes;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = lay.ranks;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (dim == 2)
    cudaLaunchKernelEx(&cfg, k_coarse_cluster<T, 2>, tab, lay, cp, fcycle, skip_pre);
  else
    cudaLaunchKernelEx(&cfg, k_coarse_cluster<T, 3>, tab, lay, cp, fcycle, skip_pre);
}

template int prepare_coarse_cluster<double>(int, size_t, int);
template int prepare_coarse_cluster<float>(int, size_t, int);
template void launch_coarse_cluster<double>(int, const LvlTable<double>*, const ClusterLayout&, const CycleParams&,
                                            int, int, size_t, cudaStream_t);
template void launch_coarse_cluster<float>(int, const LvlTable<float>*, const ClusterLayout&, const CycleParams&, int,
                                           int, size_t, cudaStream_t);

}  // namespace jmg
