// mg_coarse.cu — the coarse levels of a cycle inside one thread block, from shared memory.
//
// Below a few thousand points per level, a grid-wide launch per operator costs more in
// launch latency than in work. k_coarse_smem runs the reference's recursion
// (solver_2d.py:582-614) for every level from `lev0` down to L-2 in one block of 1024
// threads. phi and rhs of those levels live in dynamic shared memory in a compact
// layout (nx * ny * nz per level); the coefficients stay in global memory (they were
// written before the launch and are only read, through the read-only cache). The block
// loads phi/rhs of lev0 at entry and writes phi of lev0 back at exit; the deeper levels
// exist only in shared memory. The arithmetic of every point is the same as in the
// grid-wide kernels (mg_common.cuh), in the reference's order.
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

template <typename T>
struct SmemView {
  T* phi;
  T* rhs;
  int nx, ny, nz;  // compact padded extents
};

template <typename T, int DIM>
__device__ __forceinline__ T s_gs(const SmemView<T>& v, const Lvl<T>& g, int k, int j, int i) {
  const int sy = v.nx, sz = v.nx * v.ny;
  const int q = (k * v.ny + j) * v.nx + i;
  const long long p = (long long)k * g.S + (long long)j * g.P + i;
  const T* ph = v.phi;
  T s;
  if (DIM == 3) {
    s = __ldg(&g.wz[p]) * ph[q + sz];
    s = fma(__ldg(&g.wz[p - g.S]), ph[q - sz], s);
    s = fma(__ldg(&g.wy[p]), ph[q + sy], s);
  } else {
    s = __ldg(&g.wy[p]) * ph[q + sy];
  }
  s = fma(__ldg(&g.wy[p - g.P]), ph[q - sy], s);
  s = fma(__ldg(&g.wx[p]), ph[q + 1], s);
  s = fma(__ldg(&g.wx[p - 1]), ph[q - 1], s);
  s = s - v.rhs[q];
  return s * __ldg(&g.invd[p]);
}

template <typename T, int DIM>
__device__ __forceinline__ T s_defect(const SmemView<T>& v, const Lvl<T>& g, int k, int j, int i) {
  const int sy = v.nx, sz = v.nx * v.ny;
  const int q = (k * v.ny + j) * v.nx + i;
  const long long p = (long long)k * g.S + (long long)j * g.P + i;
  const T* ph = v.phi;
  T d = __ldg(&g.acc[p]) * ph[q];
  d = fma(-__ldg(&g.wx[p - 1]), ph[q - 1], d);
  d = fma(-__ldg(&g.wx[p]), ph[q + 1], d);
  d = fma(-__ldg(&g.wy[p - g.P]), ph[q - sy], d);
  d = fma(-__ldg(&g.wy[p]), ph[q + sy], d);
  if (DIM == 3) {
    d = fma(-__ldg(&g.wz[p - g.S]), ph[q - sz], d);
    d = fma(-__ldg(&g.wz[p]), ph[q + sz], d);
  }
  return d + v.rhs[q];
}

template <typename T, int DIM>
__device__ void s_sweep(const SmemView<T>& v, const Lvl<T>& g) {
  const int hx = g.mx / 2, ny = g.my - 1, nz = DIM == 3 ? g.mz - 1 : 1;
  const int n = hx * ny * nz;
  for (int color = 0; color < 2; ++color) {
    const int par = DIM == 2 ? color : (first_color_parity<3>() + color) & 1;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int r = t / hx;
      const int j = 2 + r % ny, k = DIM == 3 ? 2 + r / ny : 0;
      const int i = 2 + ((j + k + par) & 1) + 2 * (t % hx);
      if (i > g.mx) continue;
      v.phi[(k * v.ny + j) * v.nx + i] = s_gs<T, DIM>(v, g, k, j, i);
    }
    __syncthreads();
  }
}

template <typename T, int DIM>
__device__ void s_restrict(const SmemView<T>& f, const Lvl<T>& gf, const SmemView<T>& c, const Lvl<T>& gc) {
  const int n = c.nx * c.ny * c.nz;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int I = t % c.nx, J = (t / c.nx) % c.ny, K = t / (c.nx * c.ny);
    T v = T(0);
    const bool in = I >= 2 && I <= gc.mx && J >= 2 && J <= gc.my && (DIM == 2 || (K >= 2 && K <= gc.mz));
    if (in) {
      const int i = 2 * I - 1, j = 2 * J - 1, k = DIM == 3 ? 2 * K - 1 : 0;
      if (DIM == 2) {
        const T dne = s_defect<T, 2>(f, gf, 0, j + 1, i + 1);
        const T dnw = s_defect<T, 2>(f, gf, 0, j + 1, i - 1);
        const T dse = s_defect<T, 2>(f, gf, 0, j - 1, i + 1);
        const T dsw = s_defect<T, 2>(f, gf, 0, j - 1, i - 1);
        const T dc = s_defect<T, 2>(f, gf, 0, j, i);
        v = T(0.0625) * (((dne + dnw) + dse) + dsw) + T(0.25) * dc;
      } else {
        // the 12 edge-diagonal red neighbours in the reference's order (solver_3d.py:649)
        T s = s_defect<T, 3>(f, gf, k, j + 1, i + 1);
        s = s + s_defect<T, 3>(f, gf, k, j + 1, i - 1);
        s = s + s_defect<T, 3>(f, gf, k, j - 1, i + 1);
        s = s + s_defect<T, 3>(f, gf, k, j - 1, i - 1);
        s = s + s_defect<T, 3>(f, gf, k + 1, j, i + 1);
        s = s + s_defect<T, 3>(f, gf, k + 1, j, i - 1);
        s = s + s_defect<T, 3>(f, gf, k - 1, j, i + 1);
        s = s + s_defect<T, 3>(f, gf, k - 1, j, i - 1);
        s = s + s_defect<T, 3>(f, gf, k + 1, j + 1, i);
        s = s + s_defect<T, 3>(f, gf, k + 1, j - 1, i);
        s = s + s_defect<T, 3>(f, gf, k - 1, j + 1, i);
        s = s + s_defect<T, 3>(f, gf, k - 1, j - 1, i);
        v = T(0.03125) * s + T(0.125) * s_defect<T, 3>(f, gf, k, j, i);
      }
    }
    c.rhs[t] = v;
    c.phi[t] = T(0);
  }
  __syncthreads();
}

template <typename T, int DIM>
__device__ void s_prolong(const SmemView<T>& f, const Lvl<T>& gf, const SmemView<T>& c, bool diag) {
  // the coarse values are read through a Lvl view of the compact smem layout
  Lvl<T> cv;
  cv.phi = c.phi;
  cv.P = c.nx;
  cv.S = (long long)c.nx * c.ny;
  const int nx = gf.mx - 1, ny = gf.my - 1, nz = DIM == 3 ? gf.mz - 1 : 1;
  const int n = nx * ny * nz;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = 2 + t % nx, j = 2 + (t / nx) % ny, k = DIM == 3 ? 2 + t / (nx * ny) : 0;
    T v;
    const bool ok = DIM == 2 ? prolong_point2d<T>(cv, j, i, diag, &v) : prolong_point3d<T>(cv, k, j, i, diag, &v);
    if (ok) {
      const int q = (k * f.ny + j) * f.nx + i;
      f.phi[q] = f.phi[q] + v;
    }
  }
  __syncthreads();
}

// shared-memory view of level l: levels lev0..l-1 come first, phi then rhs each
template <typename T, int DIM>
__device__ __forceinline__ SmemView<T> view_of(const LvlTable<T>* tab, T* base, int lev0, int l) {
  int off = 0;
  for (int k = lev0; k < l; ++k) {
    const Lvl<T>& g = tab->l[k];
    off += 2 * (g.mx + 3) * (g.my + 3) * (DIM == 3 ? g.mz + 3 : 1);
  }
  const Lvl<T>& g = tab->l[l];
  SmemView<T> v;
  v.nx = g.mx + 3;
  v.ny = g.my + 3;
  v.nz = DIM == 3 ? g.mz + 3 : 1;
  v.phi = base + off;
  v.rhs = base + off + v.nx * v.ny * v.nz;
  return v;
}

template <typename T, int DIM>
__global__ void __launch_bounds__(1024) k_coarse_smem(const LvlTable<T>* __restrict__ tab, CycleParams cp,
                                                      int lev0, int fcycle0, int skip_pre0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* base = reinterpret_cast<T*>(smem_raw);
  // load phi and rhs of the entry level
  {
    const Lvl<T>& g = tab->l[lev0];
    const SmemView<T> v0 = view_of<T, DIM>(tab, base, lev0, lev0);
    const int n = v0.nx * v0.ny * v0.nz;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int I = t % v0.nx, J = (t / v0.nx) % v0.ny, K = t / (v0.nx * v0.ny);
      const long long p = (long long)K * g.S + (long long)J * g.P + I;
      v0.phi[t] = g.phi[p];
      v0.rhs[t] = g.rhs[p];
    }
    __syncthreads();
  }
  struct Frame {
    int lev, stage, g;
    bool fcycle, skip_pre;
  };
  Frame st[kMaxLevels + 1];
  int sp = 0;
  st[sp++] = Frame{lev0, 0, 0, fcycle0 != 0, skip_pre0 != 0};
  while (sp > 0) {
    Frame& f = st[sp - 1];
    const Lvl<T>& g = tab->l[f.lev];
    const SmemView<T> vf = view_of<T, DIM>(tab, base, lev0, f.lev);
    if (f.lev == cp.last_level) {
      for (int s = 0; s < cp.nu1 + cp.nu2; ++s) s_sweep<T, DIM>(vf, g);
      --sp;
      continue;
    }
    const SmemView<T> vc = view_of<T, DIM>(tab, base, lev0, f.lev + 1);
    if (f.stage == 0) {
      if (!f.skip_pre)
        for (int s = 0; s < cp.nu1; ++s) s_sweep<T, DIM>(vf, g);
      s_restrict<T, DIM>(vf, g, vc, tab->l[f.lev + 1]);
      f.stage = f.fcycle ? 1 : 2;
      f.g = 0;
    }
    if (f.stage == 1) {
      if (f.g < cp.gamma) {
        ++f.g;
        st[sp++] = Frame{f.lev + 1, 0, 0, true, false};
        continue;
      }
      f.stage = 2;
      f.g = 0;
    }
    if (f.stage == 2) {
      if (f.g < cp.gamma) {
        ++f.g;
        st[sp++] = Frame{f.lev + 1, 0, 0, false, false};
        continue;
      }
      f.stage = 3;
    }
    s_prolong<T, DIM>(vf, g, vc, cp.diag != 0);
    for (int s = 0; s < cp.nu2; ++s) s_sweep<T, DIM>(vf, g);
    --sp;
  }
  // write phi of the entry level back
  {
    const Lvl<T>& g = tab->l[lev0];
    const SmemView<T> v0 = view_of<T, DIM>(tab, base, lev0, lev0);
    const int n = v0.nx * v0.ny * v0.nz;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int I = t % v0.nx, J = (t / v0.nx) % v0.ny, K = t / (v0.nx * v0.ny);
      g.phi[(long long)K * g.S + (long long)J * g.P + I] = v0.phi[t];
    }
  }
}

size_t coarse_smem_bytes(int dim, const int* m0, int lev0, int last, size_t elem) {
  size_t n = 0;
  for (int l = lev0; l <= last; ++l) {
    size_t e = (size_t)((m0[0] >> l) + 3) * ((m0[1] >> l) + 3);
    if (dim == 3) e *= (size_t)((m0[2] >> l) + 3);
    n += 2 * e;
  }
  return n * elem;
}

template <typename T>
int prepare_coarse_smem(int dim, size_t bytes) {
  cudaError_t e = dim == 2 ? cudaFuncSetAttribute(k_coarse_smem<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)bytes)
                           : cudaFuncSetAttribute(k_coarse_smem<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)bytes);
  return e == cudaSuccess ? 0 : 1;
}

template <typename T>
void launch_coarse_smem(int dim, const LvlTable<T>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                        size_t smem, cudaStream_t s) {
  if (dim == 2)
    k_coarse_smem<T, 2><<<1, 1024, smem, s>>>(tab, cp, lev, fcycle, skip_pre);
  else
    k_coarse_smem<T, 3><<<1, 1024, smem, s>>>(tab, cp, lev, fcycle, skip_pre);
}

template int prepare_coarse_smem<double>(int, size_t);
template int prepare_coarse_smem<float>(int, size_t);
template void launch_coarse_smem<double>(int, const LvlTable<double>*, const CycleParams&, int, int, int, size_t,
                                         cudaStream_t);
template void launch_coarse_smem<float>(int, const LvlTable<float>*, const CycleParams&, int, int, int, size_t,
                                        cudaStream_t);

}  // namespace jmg
