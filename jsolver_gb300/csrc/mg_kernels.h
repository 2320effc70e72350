// mg_kernels.h — host-side launchers of the solver kernels (internal to libjmg).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mg_common.cuh"

namespace jmg {

// Kernel launch with programmatic stream serialisation (PDL) unless JMG_PDL=0. The
// kernel must call pdl_enter() before touching memory (mg_common.cuh).
bool pdl_enabled();
template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

struct CycleParams {
  int last_level;  // L-2: the deepest level visited (solver_2d.py:601)
  int nu1, nu2, gamma;
  int diag;        // prolongate the (even,even) points in 2D / bilinear points in 3D
};

// Scalars the device loop keeps in the workspace.
struct LoopState {
  unsigned long long dist_bits;  // max |phi_old - phi| as ordered bits (abs_bits)
  long long count;               // cycles done
  double res_norm;               // current ||r||_2 (residual stop)
  double rhs_norm;               // ||rhs||_2 over the interior (residual stop)
  double rel_res;                // res_norm / rhs_norm
  int go;                        // last loop decision
  int fault;                     // a bounded device-side wait ran out (the loop then ends)
  unsigned bar_count;            // grid barrier of the persistent middle-level kernel
                                 // (mg_mid2d.cu): arrivals, and the generation on a line
  alignas(128) unsigned bar_gen; // of its own, so that polling it does not slow the adds
};

// one full sweep (two colour passes, in place); with zero_init it starts from phi = 0
template <typename T> void launch_sweep(int dim, Lvl<T>& a, cudaStream_t s, bool zero_init = false);
// One-pass red-black sweep of a 3D level from a.phi into a.phi2, then the two pointers
// swap (mg_fused.cu); bit-identical to launch_sweep. zero_in: phi is taken as zero.
template <typename T> void launch_sweep_fused3d(Lvl<T>& a, bool zero_in, cudaStream_t s);
// mg_sweep_tma3d.cu: the same sweep for FP32 levels with its plane tiles fed by TMA copies
// (the default; JMG_SWEEP3D=regs keeps k_sweep_fused3d). false: it cannot run here (no
// tensor-map encoder or not enough shared memory), nothing was launched.
bool sweep_tma3d_ready();
bool sweep_tma3d_enabled();
bool launch_sweep_tma3d(Lvl<float>& a, bool zero_in, cudaStream_t s);
int sweep_tma3d_fault();  // reads and clears the flag of a sweep whose copies did not arrive
// The 2D one-pass sweep (tiles of 64 x 16 with a halo, mg_fused.cu), and the dispatch of
// either by dimension; levels with a second phi buffer only, no D_xy.
template <typename T> void launch_sweep_onepass2d(Lvl<T>& a, bool zero_in, cudaStream_t s);
template <typename T> void launch_sweep_onepass(int dim, Lvl<T>& a, bool zero_in, cudaStream_t s);
template <typename T> void launch_restrict_tile3d(const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s);
template <typename T> void launch_prolong_cells3d(const Lvl<T>& f, const Lvl<T>& c, int bilinear, cudaStream_t s);
template <typename T> void launch_prolong_cells2d(const Lvl<T>& f, const Lvl<T>& c, int diag, cudaStream_t s);
int fused_chunk3d(int mx, int my, int mz, int blocks_per_sm);
int fused_blocks3d(int mx, int my, int mz);
int fused_wave_permille(int mx, int my, int mz);
// mg_fusedops2d.cu: 2D operator pairs over tiles with halos; each writes f.phi2 and swaps
// f.phi / f.phi2. smooth_restrict: the last pre-sweep, then defect + restriction onto c
// (and phi_c = 0); zero_in: f.phi is zero (not read). prolong_smooth: phi += P phi_c, then
// one sweep (levels with nu2 >= 1 and no D_xy).
template <typename T> void launch_smooth_restrict2d(Lvl<T>& f, const Lvl<T>& c, bool zero_in, cudaStream_t s);
template <typename T> void launch_prolong_smooth2d(Lvl<T>& f, const Lvl<T>& c, cudaStream_t s);
void prepare_fused_ops2d();
// mg_fusedops3d.cu: the same pairs on 3D levels (7-point stencil)
template <typename T> void launch_smooth_restrict3d(Lvl<T>& f, const Lvl<T>& c, bool zero_in, cudaStream_t s);
template <typename T> void launch_prolong_smooth3d(Lvl<T>& f, const Lvl<T>& c, cudaStream_t s);
void prepare_fused_ops3d();
template <typename T>
inline void launch_smooth_restrict(int dim, Lvl<T>& f, const Lvl<T>& c, bool zero_in, cudaStream_t s) {
  if (dim == 3) launch_smooth_restrict3d<T>(f, c, zero_in, s);
  else launch_smooth_restrict2d<T>(f, c, zero_in, s);
}
template <typename T>
inline void launch_prolong_smooth(int dim, Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  if (dim == 3) launch_prolong_smooth3d<T>(f, c, s);
  else launch_prolong_smooth2d<T>(f, c, s);
}
// mg_tile2d.cu: defect + restriction with every fine defect computed once
template <typename T> void launch_restrict_tile2d(const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s);
// mg_tile2d.cu: r32 = float(rhs - L_h phi) (FP64 arithmetic) on the interior, and per-block
// sums of r^2 into parts[0 .. residual_f32_parts2d(mx, my))
int residual_f32_parts2d(int mx, int my);
void launch_residual_f32_2d(const Lvl<double>& a, float* r32, double* parts, cudaStream_t s);
template <typename T> void launch_restrict(int dim, const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s);
// the one-thread-per-coarse-point restriction (2D and 3D)
template <typename T> void launch_restrict_grid(int dim, const Lvl<T>& f, const Lvl<T>& c, cudaStream_t s);
template <typename T> void launch_prolong(int dim, const Lvl<T>& f, const Lvl<T>& c, int diag, cudaStream_t s);
template <typename T>
void launch_coarse_cycle(int dim, const LvlTable<T>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                         cudaStream_t s);
// mg_coarse.cu: the coarse sub-cycle on one thread-block cluster (rows of every level
// spread over the CTAs' shared memory)
constexpr int kMaxClusterRanks = 16;
struct ClusterLevel {
  int off;        // element offset of the level's block in every CTA's shared memory
  int nx, ny;     // padded extents along x and y
  int rp;         // row pitch in shared memory (nx rounded up to 4 elements)
  int nrows;      // rows of the level ((my+3) in 2D, (mz+3)(my+3) in 3D)
  int rpr;        // rows per CTA
  int dist;       // 1: rows spread over all CTAs; 0: the whole level lives in CTA 0
  int m[3];
};
struct ClusterLayout {
  int lev0, last, ranks;
  long long elems;  // elements of shared memory per CTA
  ClusterLevel l[kMaxLevels];
};
// m[l][axis]: resolution of level l. Returns 0 on success.
int cluster_layout(int dim, const int m[][3], int lev0, int last, int ranks, ClusterLayout* out);
// sets the kernel's shared-memory / cluster-size attributes and checks that one cluster
// of `ranks` CTAs fits on the GPU (0: usable)
template <typename T> int prepare_coarse_cluster(int dim, size_t smem_bytes, int ranks);
template <typename T>
void launch_coarse_cluster(int dim, const LvlTable<T>* tab, const ClusterLayout& lay, const CycleParams& cp,
                           int fcycle, int skip_pre, size_t smem_bytes, cudaStream_t s);
// mg_kernels.cu: FP32 2D coarse sub-cycle with every array of the coarse levels staged in
// shared memory (bytes from coarse_smem32_bytes; 0 from prepare_coarse_smem32 = usable)
size_t coarse_smem32_bytes(const int* mx, const int* my, int lev0, int last);
int prepare_coarse_smem32(size_t bytes);
void launch_coarse_smem32(const LvlTable<float>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                          size_t smem, cudaStream_t s);
// mg_coarse_staged.cu: the coarse sub-cycle on one block with every coarse array in shared
// memory, staged by bulk copies (bytes from coarse_staged_bytes, 0 = does not fit;
// prepare_coarse_staged: 0 = usable)
size_t coarse_staged_bytes(int dim, const size_t* elems, int lev0, int last, size_t elem_size, bool offdiag);
template <typename T> int prepare_coarse_staged(int dim, size_t bytes);
template <typename T>
void launch_coarse_staged(int dim, const LvlTable<T>* tab, const CycleParams& cp, int lev, int fcycle, int skip_pre,
                          size_t smem, int threads, cudaStream_t s);
// mg_mid2d.cu: the 2D middle levels (fused operator pairs between grid barriers) and the
// coarse sub-cycle (block 0, levels staged in shared memory) in one cooperative launch.
// Operation list: (kind << 12) | (flag << 8) | level, in the order of the recursion; flag
// is zero_in for kMidSR and the colour for kMidColor.
constexpr int kMaxMidOps = 4000;
struct MidOps {
  int n;
  unsigned short op[kMaxMidOps];
};
enum { kMidBlkSweep = 0, kMidBlkRestrict = 1, kMidBlkProlong = 2, kMidSR = 3, kMidPS = 4, kMidColor = 5 };
// the list of multigrid_cycle(lev) for levels lev .. coarse_start - 1 fused and the coarse
// levels on block 0; false when it exceeds kMaxMidOps
bool mid_ops(const CycleParams& cp, int coarse_start, int lev, bool fcycle, bool zero_phi, MidOps* out);
// sets the kernel's attributes; returns its dynamic shared-memory bytes (0: it cannot run:
// no cooperative launch, or one block with this much shared memory does not fit an SM)
// and the grid size (one block per SM)
template <typename T> size_t prepare_mid2d(size_t staged_bytes, int* blocks);
// stall: test mode whose first grid barrier never completes (its bounded wait runs out)
template <typename T>
cudaError_t launch_mid2d(const LvlTable<T>* tab, LoopState* st, const CycleParams& cp, int coarse_start,
                         const MidOps& ops, size_t smem, int blocks, bool stall, cudaStream_t s);
// copies a level table into device memory (the coarse kernel reads it from there)
template <typename T> void launch_store_table(const LvlTable<T>& tab, LvlTable<T>* dst, cudaStream_t s);

// mg_aux.cu
struct Box {  // padded extents of one level
  int nx, ny, nz;  // m+3 per axis (nz = 1 in 2D)
  int P;
  long long S;
};
void launch_copy_in(const Box& b, const double* src_dense, double* dst, int zero_frame, cudaStream_t s);
void launch_copy_out(const Box& b, const double* src, double* dst_dense, cudaStream_t s);
void launch_do_bcs_dense(int dim, const int32_t* shape, double* arr, cudaStream_t s);
// max |a - b| over the padded box into st->dist_bits (after zeroing it), then a <- b.
void launch_distance_snapshot(const Box& b, double* old_phi, const double* phi, LoopState* st, cudaStream_t s);
// partial sums of squares of the defect (or of rhs when phi == nullptr) over the interior
template <typename T>
void launch_residual_partials(int dim, const Lvl<T>& a, const T* phi_or_null, double* partials, int nparts,
                              cudaStream_t s, float* r32 = nullptr);
int residual_num_parts(int dim, const Box& b);
// device-side loop decisions
void launch_loop_init(LoopState* st, const double* partials, int nparts, int mode, double rtol,
                      long long max_iters, unsigned long long cond_handle, cudaStream_t s);
void launch_loop_step(LoopState* st, const double* partials, int nparts, int mode, double eps, double rtol,
                      long long max_iters, unsigned long long cond_handle, cudaStream_t s);
void launch_rhs_norm(LoopState* st, const double* partials, int nparts, cudaStream_t s);
void launch_rel_residual_out(const LoopState* st, const double* partials, int nparts, double* out, cudaStream_t s);
void launch_count_out(const LoopState* st, long long* out, cudaStream_t s);
void launch_dense_residual(int dim, const Lvl<double>& a, const Box& b, double* d_dense, cudaStream_t s);
void launch_copy_coeff(const Box& b, const double* src, double* dst_dense, cudaStream_t s);

// mixed precision helpers (mg_aux.cu)
// r32 = rhs - L_h phi (FP64 arithmetic, FP32 result) on the interior, zero frame.
void launch_residual_to_f32(int dim, const Lvl<double>& a, float* r32, cudaStream_t s);
// phi += e32 on the interior; e32 untouched.
void launch_add_correction(int dim, const Lvl<double>& a, const float* e32, cudaStream_t s);
void launch_zero_f32(const Box& b, float* x, cudaStream_t s);
void launch_convert_f32(const Box& b, const double* src, float* dst, cudaStream_t s);

// mg_krylov.cu: FCG(1) around the cycle (outer = FCG)
int fcg_num_parts();                                // partial-sum slots to reserve
int fcg_parts_used(int dim, const Lvl<double>& a);  // partials a solve of this size writes
// rho = rhs - L x (x = a.phi), d = q = 0, r32 = float(rho) (nullable); partials of rho^2
void launch_fcg_init(int dim, const Lvl<double>& a, double* rho, double* d, double* q, float* r32, double* parts,
                     cudaStream_t s);
// mixed precision (FP32 directions d, q; FP64 x and true residual): init and one step
// (dots, directions, x update, residual: 4 launches)
void launch_fcg32_init(int dim, const Lvl<double>& a, float* r32, float* d, float* q, double* parts, cudaStream_t s);
void launch_fcg32_iter(int dim, const Lvl<double>& a, const Lvl<float>& a32, const float* z, float* d, float* q,
                       float* r32, double* parts_dots, double* parts_dir, double* parts_res, cudaStream_t s);
// one FCG step after the preconditioner produced z: dots, direction, update (3 launches)
template <typename TZ>
void launch_fcg_iter(int dim, const Lvl<double>& a, const TZ* z, double* d, double* q, double* rho, float* r32,
                     double* parts_dots, double* parts_dir, double* parts_res, cudaStream_t s);

// mg_driver.cu: records the message jmg_last_error() returns; returns code
int set_error_message(int code, const char* msg);

// mg_hierarchy.cu
struct HierInputs {
  const double* lam; double lam_scalar;
  const double* D[3]; double D_scalar[3];
  int scalar_D;     // all D components scalar
  int scalar_lam;
  const double* Dxy = nullptr;  // 2D off-diagonal D (array D only), or nullptr
};
// Builds wx, wy, (wz), acc, invd of level l (and the averaged D arrays of level l in 3D).
// dprev: averaged D of level l-1 (3D, l >= 2), or nullptr.
void launch_hierarchy_level(int dim, int level, const Lvl<double>& a, const Box& b, const Box& b0,
                            const HierInputs& in, const double* idel, const double* sq_idel, double* const* d_cur,
                            const double* const* d_prev, const Box& bprev, cudaStream_t s);

}  // namespace jmg
