// mg_kernels.cu — sm_103a kernels of the multigrid cycle (2D and 3D, FP64 and FP32).
//
// Grid-wide kernels, one launch per operator, run the fine levels:
//   k_sweep_color   one colour of the red-black Gauss-Seidel sweep (solver_2d.py:670-692,
//                   solver_3d.py:679-706); two launches make one sweep
//   k_restrict      defect + red-point restriction onto level+1, also zeroes phi_{l+1}
//                   (solver_2d.py:607-608, 616-647; solver_3d.py:613-614, 622-652)
//   k_prolong       phi += P(phi_c) (solver_2d.py:612, 649-668; solver_3d.py:618, 654-677)
// The coarse levels (few thousand points) run inside one thread block: k_coarse_cycle
// executes the reference's recursion (solver_2d.py:582-614) from a given level down to
// level L-2 with __syncthreads between operators, so a whole V/W/F sub-cycle is one launch.
#include <cstdlib>
#include <cstring>

#include "mg_block.cuh"
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_dual.cuh"

namespace jmg {

// ------------------------------------------------------------------------------------
// grid-wide operators
// ------------------------------------------------------------------------------------

// 2D: blockDim (64, 4); x walks the points of one colour in a row, y walks rows. With
// zero_other, the other colour is taken as zero without being read: the first colour
// pass of a sweep from a zero initial guess (a refinement step's correction).
// With D_xy the two sub-lattices of a colour neighbour each other diagonally, so the
// reference's order matters: row_par >= 0 restricts the pass to the rows of that parity
// (one sub-lattice), and four passes make a sweep (solver_2d.py:684).
template <typename T>
__global__ void k_sweep_color2d(Lvl<T> a, int color, int zero_other, int row_par) {
  pdl_enter();
  const int r = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = row_par < 0 ? r + 2 : 2 + row_par + 2 * r;
  if (i > a.my) return;
  const int j = 2 + ((i + color) & 1) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (j > a.mx) return;
  const long long p = (long long)i * a.P + j;
  // with all neighbours zero, (0 - rhs) / A_cc is what the full expression gives
  a.phi[p] = zero_other ? (T(0) - a.rhs[p]) * a.invd[p] : gs_point2d<T>(a, p);
}

// 3D: blockDim (64, 4, 1); grid z walks planes.
template <typename T>
__global__ void k_sweep_color3d(Lvl<T> a, int color, int zero_other) {
  pdl_enter();
  const int k = blockIdx.z + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (j > a.my || k > a.mz) return;
  // first colour in 3D: i+j+k odd (color 0); second: even
  const int par = (first_color_parity<3>() + color) & 1;
  const int i = 2 + ((j + k + par) & 1) + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (i > a.mx) return;
  const long long p = (long long)k * a.S + (long long)j * a.P + i;
  a.phi[p] = zero_other ? (T(0) - a.rhs[p]) * a.invd[p]
                        : gs_point3d<T>(a.phi, a.rhs, a.wx, a.wy, a.wz, a.invd, p, a.P, a.S);
}

// Over the full padded coarse array: phi_c = 0, rhs_c = restricted defect inside, 0 on the frame.
template <typename T>
__global__ void k_restrict2d(Lvl<T> f, Lvl<T> c) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I > c.mx + 2 || J > c.my + 2) return;
  const long long q = (long long)J * c.P + I;
  c.phi[q] = T(0);
  T v = T(0);
  if (J >= 2 && J <= c.my && I >= 2 && I <= c.mx) v = restrict_point2d<T>(f, J, I);
  c.rhs[q] = v;
}

template <typename T>
__global__ void k_restrict3d(Lvl<T> f, Lvl<T> c) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I > c.mx + 2 || J > c.my + 2) return;
  const long long q = (long long)K * c.S + (long long)J * c.P + I;
  c.phi[q] = T(0);
  T v = T(0);
  if (K >= 2 && K <= c.mz && J >= 2 && J <= c.my && I >= 2 && I <= c.mx) v = restrict_point3d<T>(f, K, J, I);
  c.rhs[q] = v;
}

template <typename T>
__global__ void k_prolong2d(Lvl<T> f, Lvl<T> c, int diag) {
  pdl_enter();
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (i > f.my || j > f.mx) return;
  T v;
  if (prolong_point2d<T>(c, i, j, diag != 0, &v)) {
    const long long p = (long long)i * f.P + j;
    f.phi[p] = f.phi[p] + v;
  }
}

template <typename T>
__global__ void k_prolong3d(Lvl<T> f, Lvl<T> c, int bilinear) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > f.mx || j > f.my) return;
  T v;
  if (prolong_point3d<T>(c, k, j, i, bilinear != 0, &v)) {
    const long long p = (long long)k * f.S + (long long)j * f.P + i;
    f.phi[p] = f.phi[p] + v;
  }
}

// ------------------------------------------------------------------------------------
// single-block coarse cycle
// ------------------------------------------------------------------------------------

// The level table (~2 KB) is copied into shared memory first: every frame of the cycle
// reads its level's pointers and sizes, and from the global table each of those reads
// was an L2 round trip in front of the frame's first pass.
template <typename T, int DIM>
__global__ void __launch_bounds__(1024) k_coarse_cycle(const LvlTable<T>* tab, CycleParams cp, int lev, int fcycle,
                                                      int skip_pre, CoarseOps ops) {
  pdl_enter();
  __shared__ LvlTable<T> stab;
  __shared__ CoarseOps sops;
  {
    const int n = (int)(sizeof(LvlTable<T>) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(tab);
    int* dst = reinterpret_cast<int*>(&stab);
    for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
  }
  stage_coarse_ops(ops, &sops);
  __syncthreads();
  if (sops.n > 0) blk_run<T, DIM>(&stab, cp, &sops);
  else blk_cycle<T, DIM>(&stab, cp, lev, fcycle != 0, skip_pre != 0);
}

// FP32 2D coarse sub-cycle from shared memory. Every array of levels lev0 .. last (phi,
// rhs, wx, wy, acc, invd; row pitch rp = nx rounded up to 4 floats) is staged in dynamic
// shared memory with 16-byte loads, the recursion of blk_cycle then runs on shared-memory
// views of the levels, and phi of lev0 is written back. Each pass of the cycle then costs
// shared-memory latency instead of an L2 round trip, but the staging itself (~150 KB at
// 2D 1024^2 per launch) costs more than that saves, so it is opt-in (JMG_COARSE32=smem).
constexpr int kSmem32Max = 200 * 1024;

__host__ __device__ inline int smem32_rp(int mx) { return (mx + 3 + 3) & ~3; }

size_t coarse_smem32_bytes(const int* mx, const int* my, int lev0, int last) {
  size_t n = 0;
  for (int l = lev0; l <= last; ++l) n += (size_t)6 * smem32_rp(mx[l]) * (my[l] + 3);
  return n * sizeof(float);
}

__global__ void __launch_bounds__(1024) k_coarse_smem32(const LvlTable<float>* tab, CycleParams cp, int lev0,
                                                       int fcycle, int skip_pre) {
  pdl_enter();
  extern __shared__ __align__(16) float sm32[];
  __shared__ LvlTable<float> st;
  if (threadIdx.x == 0) {
    size_t off = 0;
    for (int l = lev0; l <= cp.last_level; ++l) {
      Lvl<float> v = tab->l[l];
      const int rp = smem32_rp(v.mx), ny = v.my + 3;
      const size_t n = (size_t)rp * ny;
      v.phi = sm32 + off;
      v.rhs = v.phi + n;
      v.wx = v.rhs + n;
      v.wy = v.wx + n;
      v.acc = v.wy + n;
      v.invd = v.acc + n;
      v.wz = nullptr;
      v.xll = v.xrl = v.xlr = v.xrr = nullptr;
      v.P = rp;
      v.S = (long long)n;
      st.l[l] = v;
      off += 6 * n;
    }
  }
  __syncthreads();
  // copy-in: every thread issues four 16-byte loads before it stores them, so a level's
  // arrays arrive in a few L2 round trips rather than one per loop iteration
  for (int l = lev0; l <= cp.last_level; ++l) {
    const Lvl<float>& g = tab->l[l];
    const Lvl<float>& v = st.l[l];
    const int cpr = v.P / 4, ny = v.my + 3, n = cpr * ny;
    const float* src[6] = {g.phi, g.rhs, g.wx, g.wy, g.acc, g.invd};
    float* dst[6] = {v.phi, v.rhs, v.wx, v.wy, v.acc, v.invd};
    for (int a = l == lev0 ? 0 : 2; a < 6; ++a)
      for (int t0 = threadIdx.x; t0 < n; t0 += 4 * blockDim.x) {
        float4 w[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * blockDim.x;
          if (t < n) {
            const int j = t / cpr, e = (t - j * cpr) * 4;
            w[u] = __ldcg(reinterpret_cast<const float4*>(src[a] + (long long)j * g.P + e));
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * blockDim.x;
          if (t < n) {
            const int j = t / cpr, e = (t - j * cpr) * 4;
            *reinterpret_cast<float4*>(dst[a] + j * v.P + e) = w[u];
          }
        }
      }
  }
  __syncthreads();
  blk_cycle<float, 2>(&st, cp, lev0, fcycle != 0, skip_pre != 0);
  {
    const Lvl<float>& g = tab->l[lev0];
    const Lvl<float>& v = st.l[lev0];
    const int nx = v.mx + 3, n = nx * (v.my + 3);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int j = t / nx, i = t - j * nx;
      g.phi[(long long)j * g.P + i] = v.phi[j * v.P + i];
    }
  }
}

int prepare_coarse_smem32(size_t bytes) {
  return cudaFuncSetAttribute(k_coarse_smem32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
                 cudaSuccess
             ? 0
             : 1;
}

void launch_coarse_smem32(const LvlTable<float>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                          size_t smem, cudaStream_t s) {
  launch_k(k_coarse_smem32, dim3(1), dim3(1024), smem, s, tab, cp, lev, fcycle, skip_pre);
}

template <typename T>
__global__ void k_store_table(LvlTable<T> tab, LvlTable<T>* dst) {
  const int n = sizeof(LvlTable<T>) / sizeof(int);
  const int* src = reinterpret_cast<const int*>(&tab);
  int* d = reinterpret_cast<int*>(dst);
  for (int k = threadIdx.x; k < n; k += blockDim.x) d[k] = src[k];
}

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------

static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// One full sweep: the red colour pass, then the black one, in place (a colour pass reads
// only the other colour, so it needs no second buffer). With zero_init the sweep starts
// from phi = 0 (the red pass does not read phi). a.phi holds the result on return.
template <typename T>
void launch_sweep(int dim, Lvl<T>& a, cudaStream_t s, bool zero_init) {
  if (dim == 2 && a.xll) {
    // 9-point stencil: sub-lattices (0,0), (1,1), (0,1), (1,0) of the reference
    // (odd/odd, even/even, even-row/odd-column, odd-row/even-column), one pass each
    if (zero_init) cudaMemsetAsync(a.phi, 0, (size_t)a.P * (a.my + 3) * sizeof(T), s);
    const int colour[4] = {0, 0, 1, 1}, rpar[4] = {1, 0, 0, 1};
    for (int q = 0; q < 4; ++q) {
      dim3 b(64, 4), g(cdiv(a.mx / 2, 64), cdiv((a.my - 1 + 1) / 2, 4));
      launch_k(k_sweep_color2d<T>, g, b, 0, s, a, colour[q], 0, rpar[q]);
    }
    return;
  }
  for (int color = 0; color < 2; ++color) {
    const int zero = (zero_init && color == 0) ? 1 : 0;
    if (dim == 2) {
      dim3 b(64, 4), g(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4));
      launch_k(k_sweep_color2d<T>, g, b, 0, s, a, color, zero, -1);
    } else {
      dim3 b(64, 4, 1), g(cdiv(a.mx / 2, 64), cdiv(a.my - 1, 4), a.mz - 1);
      launch_k(k_sweep_color3d<T>, g, b, 0, s, a, color, zero);
    }
  }
}

template <typename T>
void launch_restrict(int dim, const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  if (dim == 2 && !f.xll) {
    launch_restrict_tile2d<T>(f, c, s);
  } else if (dim == 2) {
    dim3 b(32, 8), g(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8));
    launch_k(k_restrict2d<T>, g, b, 0, s, f, c);
  } else {
    // the tiled form (mg_tile3d.cu) unless JMG_RESTRICT3D=grid asks for one thread per
    // coarse point; both give the same bits
    const char* e = getenv("JMG_RESTRICT3D");
    if (!(e && std::strcmp(e, "grid") == 0)) {
      launch_restrict_tile3d<T>(f, c, s);
      return;
    }
    dim3 b(32, 8, 1), g(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8), c.mz + 3);
    launch_k(k_restrict3d<T>, g, b, 0, s, f, c);
  }
}

// Defect + restriction with one thread per coarse point (the grid form of launch_restrict
// in 2D and 3D; the tiled forms give the same bits for FP64 and FP32).
template <typename T>
void launch_restrict_grid(int dim, const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  if (dim == 2) {
    dim3 b(32, 8), g(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8));
    launch_k(k_restrict2d<T>, g, b, 0, s, f, c);
  } else {
    dim3 b(32, 8, 1), g(cdiv(c.mx + 3, 32), cdiv(c.my + 3, 8), c.mz + 3);
    launch_k(k_restrict3d<T>, g, b, 0, s, f, c);
  }
}

template <typename T>
void launch_prolong(int dim, const Lvl<T>& f, const Lvl<T>& c, int diag, cudaStream_t s) {
  if (dim == 2) {
    // by coarse cells (mg_tile2d.cu) unless JMG_PROLONG2D=grid; the same bits
    const char* e2 = getenv("JMG_PROLONG2D");
    if (!(e2 && std::strcmp(e2, "grid") == 0)) {
      launch_prolong_cells2d<T>(f, c, diag, s);
      return;
    }
    dim3 b(64, 4), g(cdiv(f.mx - 1, 64), cdiv(f.my - 1, 4));
    launch_k(k_prolong2d<T>, g, b, 0, s, f, c, diag);
  } else {
    // by coarse cells (mg_tile3d.cu) unless JMG_PROLONG3D=grid asks for one thread per
    // fine point; both give the same bits
    const char* e = getenv("JMG_PROLONG3D");
    if (!(e && std::strcmp(e, "grid") == 0)) {
      launch_prolong_cells3d<T>(f, c, diag, s);
      return;
    }
    dim3 b(64, 4, 1), g(cdiv(f.mx - 1, 64), cdiv(f.my - 1, 4), f.mz - 1);
    launch_k(k_prolong3d<T>, g, b, 0, s, f, c, diag);
  }
}

template <typename T>
void launch_coarse_cycle(int dim, const LvlTable<T>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                         cudaStream_t s) {
  const CoarseOps ops = coarse_ops(cp, lev, fcycle != 0, skip_pre != 0);
  if (dim == 2)
    launch_k(k_coarse_cycle<T, 2>, dim3(1), dim3(1024), 0, s, tab, cp, lev, fcycle, skip_pre, ops);
  else
    launch_k(k_coarse_cycle<T, 3>, dim3(1), dim3(1024), 0, s, tab, cp, lev, fcycle, skip_pre, ops);
}

template <typename T>
void launch_store_table(const LvlTable<T>& tab, LvlTable<T>* dst, cudaStream_t s) {
  k_store_table<T><<<1, 128, 0, s>>>(tab, dst);
}

#define JMG_INST(T)                                                                               \
  template void launch_sweep<T>(int, Lvl<T>&, cudaStream_t, bool);                                \
  template void launch_restrict<T>(int, const Lvl<T>&, const Lvl<T>&, cudaStream_t);              \
  template void launch_prolong<T>(int, const Lvl<T>&, const Lvl<T>&, int, cudaStream_t);          \
  template void launch_coarse_cycle<T>(int, const LvlTable<T>*, const CycleParams&, int, int, int, cudaStream_t); \
  template void launch_store_table<T>(const LvlTable<T>&, LvlTable<T>*, cudaStream_t);
JMG_INST(double)
JMG_INST(float)
#undef JMG_INST
template void launch_restrict_grid<double>(int, const Lvl<double>&, const Lvl<double>&, cudaStream_t);
// the forward-mode solve (mg_tangent.cu): the same kernels over dual numbers
template void launch_sweep<Dual>(int, Lvl<Dual>&, cudaStream_t, bool);
template void launch_restrict_grid<Dual>(int, const Lvl<Dual>&, const Lvl<Dual>&, cudaStream_t);
template void launch_coarse_cycle<Dual>(int, const LvlTable<Dual>*, const CycleParams&, int, int, int, cudaStream_t);
template void launch_store_table<Dual>(const LvlTable<Dual>&, LvlTable<Dual>*, cudaStream_t);

}  // namespace jmg
