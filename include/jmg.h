/*
 * jmg.h — C ABI of the GB300 geometric-multigrid solver (jsolver_gb300).
 *
 * Drop-in boundary for davef96/jsolver's solve path. The reference's public entry
 * points are the jit-compiled functions
 *     solve_2d(grid_x, grid_y, phi, rhs, lam, D_xx, D_yy, *, D_xy, fixed, epsilon,
 *              gamma, fcycle, skip_pre, nu1, nu2, max_iters_outer, max_iters_inner)
 *         -> (phi, count)                                   jsolver/solver_2d.py:196-236
 *     solve_3d(grid_x, grid_y, grid_z, phi, rhs, lam, D_xx, D_yy, D_zz, *, fixed, ...)
 *                                                           jsolver/solver_3d.py:196-237
 * and the Solver_2D / Solver_3D methods below them (solver_2d.py:238-692,
 * solver_3d.py:239-706). Each declaration below names the reference interface it
 * replaces.
 *
 * Conventions
 *  - All arrays are float64 device pointers in the reference's padded layout: 2D
 *    row-major [y][x] of shape (my+3, mx+3); 3D [z][y][x] of shape (mz+3, my+3, mx+3)
 *    (solver_3d.py:210-212). A NULL coefficient pointer selects the scalar argument
 *    next to it (the reference's "scalar lam / scalar D" forms).
 *  - The caller owns every buffer, including the workspace. A JmgPlan is a host
 *    object created and destroyed by the caller; it caches the captured CUDA graph of
 *    the cycle loop for the pointers it was last run with.
 *  - Every call is asynchronous on the given stream and returns a status code
 *    (JMG_OK or a JMG_ERR_*); nothing throws across the ABI. jmg_last_error() gives
 *    the message of the last failure on the calling thread. Validation errors carry
 *    the reference's ValueError messages (solver_2d.py:292-321, 449-453).
 *  - Dynamic mode needs no host synchronisation: the cycle count is written to the
 *    device int64 pointed to by count_out.
 */
#ifndef JMG_H
#define JMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* jmg_stream_t; /* same type as cudaStream_t */

enum {
  JMG_OK = 0,
  JMG_ERR_VALUE = 1,     /* invalid argument: the reference raises ValueError */
  JMG_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  JMG_ERR_WORKSPACE = 3, /* workspace missing or too small */
  JMG_ERR_TIMEOUT = 4    /* a bounded device-side wait ran out: the solve's result is void,
                            the CUDA context stays usable (jmg_solve_check) */
};

enum { JMG_STOP_DISTANCE = 0, JMG_STOP_RESIDUAL = 1 };
enum { JMG_PREC_FP64 = 0, JMG_PREC_MIXED = 1 };
enum { JMG_OUTER_RICHARDSON = 0, JMG_OUTER_FCG = 1 };

/* Geometry: the fields of grid_1D the solver reads (jsolver/grid_1d.py:82-114). */
typedef struct JmgGrid {
  int32_t ndim;         /* 2 or 3 */
  int32_t m[3];         /* resolution per axis x, y, z (grid_1D.mx); z unused in 2D */
  double idel[3];       /* 1/h per axis (grid_1D.idel) */
  int32_t is_linear[3]; /* grid_1D.is_linear */
} JmgGrid;

/* Solver configuration: the static arguments of solve_2d/solve_3d (solver_2d.py:197),
 * plus the stopping rule and precision of this library's extensions. */
typedef struct JmgConfig {
  int32_t fixed;           /* 1: exactly max_iters_outer cycles (fori_loop, solver_2d.py:461-463) */
  int32_t gamma;           /* recursive calls per level: 1 = V, 2 = W */
  int32_t fcycle;          /* F-cycle (solver_2d.py:609-610) */
  int32_t skip_pre;        /* pre-smooth once before the loop, not per cycle at level 0 */
  int32_t nu1, nu2;        /* pre-/post-smoothing sweeps */
  int64_t max_iters_outer; /* cycle limit (count in fixed mode) */
  int64_t max_iters_inner; /* accepted for API parity; unused, as in the reference */
  double epsilon;          /* distance threshold of the dynamic loop (solver_2d.py:465-467) */
  int32_t stop;            /* JMG_STOP_DISTANCE (reference) or JMG_STOP_RESIDUAL */
  double rtol;             /* relative-residual target for JMG_STOP_RESIDUAL */
  int32_t precision;       /* JMG_PREC_FP64 or JMG_PREC_MIXED (FP32 cycles, FP64 refinement) */
  int32_t inner_cycles;    /* FP32 cycles per refinement step (JMG_PREC_MIXED) */
  int32_t outer;           /* JMG_OUTER_RICHARDSON (reference: phi += cycle correction) or
                              JMG_OUTER_FCG (the cycle preconditions flexible CG; needs
                              JMG_STOP_RESIDUAL or fixed; no reference counterpart) */
  int32_t off_diag;        /* 1: solves pass D_xy with array D (2D 9-point stencil,
                              solver_2d.py:410-416); the workspace then holds the diagonal
                              couplings. jmg_solve2d_f64 sets it from its coefficients. */
} JmgConfig;

/* Coefficients of one solve: lam, D_xx, D_yy (, D_zz) and optional D_xy. */
typedef struct JmgCoeffs {
  const double* lam; double lam_scalar;
  const double* D[3]; double D_scalar[3]; /* D_xx, D_yy, D_zz */
  const double* D_xy;                     /* 2D off-diagonal component or NULL */
} JmgCoeffs;

typedef struct JmgPlan JmgPlan;

/* Fills cfg with the reference defaults (solver_2d.py:197): dynamic, epsilon 1e-12,
 * gamma 1, no F-cycle, no skip_pre, nu1 = nu2 = 1, max_iters = int32 max. */
void jmg_config_default(JmgConfig* cfg);

/* Validates grid and configuration and lays out the level hierarchy
 * (Solver_2D.__init__ / compute_shapes / compute_idel, solver_2d.py:247-324;
 * solver_3d.py:248-336). Raises the reference's messages as JMG_ERR_VALUE. */
int jmg_plan_create(JmgPlan** plan, const JmgGrid* grid, const JmgConfig* cfg);
int jmg_plan_destroy(JmgPlan* plan);
size_t jmg_plan_workspace_bytes(const JmgPlan* plan);
int jmg_plan_levels(const JmgPlan* plan);

/* Full solve (Solver_2D.solve / Solver_3D.solve, solver_2d.py:423-479,
 * solver_3d.py:431-486). phi0 and phi_out may alias. count_out: device int64. */
int jmg_solve(JmgPlan* plan, const double* phi0, const double* rhs, const JmgCoeffs* coeffs,
              double* phi_out, int64_t* count_out, void* workspace, size_t workspace_bytes,
              jmg_stream_t stream);

/* Element strides between consecutive problems of a batch, per coefficient array; 0 means
 * the array is shared by every problem. Scalars (NULL arrays) ignore their stride. */
typedef struct JmgBatchStrides {
  int64_t lam;
  int64_t D[3];
  int64_t D_xy;
} JmgBatchStrides;

/* Workspace of a batched solve that runs `lanes` problems side by side (at most 32):
 * lanes x the plan's workspace, each slice aligned. */
size_t jmg_batched_workspace_bytes(const JmgPlan* plan, int32_t lanes);

/* batch independent solves of one plan (jax.vmap of solve_2d / solve_3d in the
 * reference's variational-inference use, README.md:107, examples/benchmark.py:1109-1230).
 * phi0, rhs and phi_out hold batch dense padded arrays back to back; coefficient
 * pointers address problem 0 and advance by strides per problem. counts_out: device
 * int64[batch] (or NULL). The workspace's size sets the number of lanes
 * (workspace_bytes / jmg_batched_workspace_bytes(plan, 1), at most 32 and at most batch);
 * the lanes run on the plan's own streams, forked from and joined back to `stream`.
 * Each problem's phi and count equal those of jmg_solve on it alone. */
int jmg_solve_batched(JmgPlan* plan, int32_t batch, const double* phi0, const double* rhs,
                      const JmgCoeffs* coeffs, const JmgBatchStrides* strides, double* phi_out,
                      int64_t* counts_out, void* workspace, size_t workspace_bytes,
                      jmg_stream_t stream);

/* One-shot form of jmg_solve for 2D / 3D (creates and destroys a plan). */
int jmg_solve2d_f64(const JmgGrid* grid, const JmgConfig* cfg, const double* phi0,
                    const double* rhs, const JmgCoeffs* coeffs, double* phi_out,
                    int64_t* count_out, void* workspace, size_t workspace_bytes,
                    jmg_stream_t stream);
int jmg_solve3d_f64(const JmgGrid* grid, const JmgConfig* cfg, const double* phi0,
                    const double* rhs, const JmgCoeffs* coeffs, double* phi_out,
                    int64_t* count_out, void* workspace, size_t workspace_bytes,
                    jmg_stream_t stream);

/* Coefficient hierarchy into the workspace (compute_discretization and the D / lambda
 * hierarchies, solver_2d.py:326-421; solver_3d.py:338-429). */
int jmg_build_hierarchy(JmgPlan* plan, const JmgCoeffs* coeffs, void* workspace,
                        size_t workspace_bytes, jmg_stream_t stream);

/* Operator entry points on dense padded arrays of one level; they use the hierarchy
 * built by jmg_build_hierarchy in the same workspace.
 *  jmg_op_sweep:    red_black_gauss_seidel (solver_2d.py:670-692; solver_3d.py:679-706),
 *                   in place on phi.
 *  jmg_op_restrict: defect + restriction (solver_2d.py:616-647; solver_3d.py:622-652);
 *                   writes the level+1 array rhs_c.
 *  jmg_op_prolong:  phi += prolongate(phi_c) (solver_2d.py:612, 649-668;
 *                   solver_3d.py:618, 654-677), in place on phi.
 *  jmg_op_residual: defect field d = rhs - L_h phi on the interior (defect before
 *                   restriction, solver_2d.py:632-642), zero frame.
 *  jmg_op_coeff:    copies one coefficient array of a level out of the workspace
 *                   (which: 0 = A_cc, 1 = x-face, 2 = y-face, 3 = z-face), dense padded. */
int jmg_op_sweep(JmgPlan* plan, int level, double* phi, const double* rhs, void* workspace,
                 size_t workspace_bytes, jmg_stream_t stream);
int jmg_op_restrict(JmgPlan* plan, int level, const double* phi, const double* rhs,
                    double* rhs_c, void* workspace, size_t workspace_bytes, jmg_stream_t stream);
int jmg_op_prolong(JmgPlan* plan, int level, double* phi, const double* phi_c, void* workspace,
                   size_t workspace_bytes, jmg_stream_t stream);
int jmg_op_residual(JmgPlan* plan, int level, const double* phi, const double* rhs, double* d,
                    void* workspace, size_t workspace_bytes, jmg_stream_t stream);
int jmg_op_coeff(JmgPlan* plan, int level, int which, double* out, void* workspace,
                 size_t workspace_bytes, jmg_stream_t stream);

/* Relative residual ||rhs - L_h phi||_2 / ||rhs||_2 over interior indices 2..m, FP64,
 * written to the device double *out (the measure the benchmark stops on). */
int jmg_rel_residual(JmgPlan* plan, const double* phi, const double* rhs, double* out,
                     void* workspace, size_t workspace_bytes, jmg_stream_t stream);

/* do_BCs(arr) with rim 1 and zero values (boundary_handler_2d.py:3-30,
 * boundary_handler_3d.py:3-35), in place on a dense padded device array. */
int jmg_do_bcs(int ndim, const int32_t* shape, double* arr, jmg_stream_t stream);

/* Reverse mode of the fixed-mode 2D solve: given phi_bar = dL/dphi_n for phi_n =
 * solve_2d(..., fixed=True, max_iters_outer=n), writes the vector-Jacobian products
 * dL/dphi0, dL/drhs, dL/dlam, dL/dD_xx, dL/dD_yy (dense padded arrays). Replaces
 * jax.vjp of the reference's fixed mode (solver_2d.py:18-26, 461-463; exercised in
 * tests/test_solver_2d.py:200-207). lam and D must be arrays. Needs the plan's workspace
 * and an adjoint workspace of jmg_adjoint_workspace_bytes(plan) bytes (per-cycle
 * checkpoints of phi plus per-operator snapshots of one cycle, which is recomputed). */
size_t jmg_adjoint_workspace_bytes(const JmgPlan* plan);
int jmg_solve_fixed_vjp(JmgPlan* plan, const double* phi0, const double* rhs, const JmgCoeffs* coeffs,
                        const double* phi_bar, double* phi0_bar, double* rhs_bar, double* lam_bar,
                        double* Dxx_bar, double* Dyy_bar, void* workspace, size_t workspace_bytes,
                        void* adjoint_workspace, size_t adjoint_workspace_bytes, jmg_stream_t stream);
/* Reverse mode of the fixed-mode solve in 2D and 3D, with the 5-, 7- or 9-point stencil:
 * jax.vjp of solve_2d / solve_3d with fixed = True (solver_2d.py:461-463, solver_3d.py:
 * 468-470). D_bar holds one output per axis (dL/dD_xx, dL/dD_yy[, dL/dD_zz]); Dxy_bar is
 * dL/dD_xy for a plan created with off_diag (NULL otherwise). The other arguments are those
 * of jmg_solve_fixed_vjp, which is this function for 2D plans without D_xy. */
int jmg_solve_fixed_vjp_nd(JmgPlan* plan, const double* phi0, const double* rhs, const JmgCoeffs* coeffs,
                           const double* phi_bar, double* phi0_bar, double* rhs_bar, double* lam_bar,
                           double* const* D_bar, double* Dxy_bar, void* workspace, size_t workspace_bytes,
                           void* adjoint_workspace, size_t adjoint_workspace_bytes, jmg_stream_t stream);

/* Forward mode of the solve (jax.jvp through solve_2d / solve_3d: through the fixed
 * fori_loop, solver_2d.py:461-463, and through the dynamic while_loop, solver_2d.py:465-477,
 * whose cycle count follows the primal's distance test and is not differentiated; the same
 * in solver_3d.py:468-477). Writes phi and its tangent phi_dot for the tangents phi0_dot,
 * rhs_dot and the coefficient tangents coeffs_dot (lam, D components and, with a plan
 * created with off_diag, D_xy: arrays where coeffs has arrays, scalars where it has
 * scalars). 2D and 3D, 5-, 7- and 9-point stencils, V/W/F cycles, skip_pre, any nu1/nu2;
 * the reference's FP64 iteration (precision fp64, outer richardson) with fixed = 1 or the
 * distance stop. phi and the cycle count equal jmg_solve's bit for bit. count_out: device
 * int64 or NULL. The dynamic loop reads the device's loop decision back after every cycle.
 * tangent_workspace: jmg_tangent_workspace_bytes(plan) bytes, 256-byte aligned (the
 * tangent coefficient hierarchy and the dual-number level arrays). */
size_t jmg_tangent_workspace_bytes(const JmgPlan* plan);
int jmg_solve_jvp(JmgPlan* plan, const double* phi0, const double* rhs, const JmgCoeffs* coeffs,
                  const double* phi0_dot, const double* rhs_dot, const JmgCoeffs* coeffs_dot, double* phi_out,
                  double* phi_dot_out, int64_t* count_out, void* workspace, size_t workspace_bytes,
                  void* tangent_workspace, size_t tangent_workspace_bytes, jmg_stream_t stream);
/* jmg_solve_jvp for a plan with fixed = 1 (no count output). */
int jmg_solve_fixed_jvp(JmgPlan* plan, const double* phi0, const double* rhs, const JmgCoeffs* coeffs,
                        const double* phi0_dot, const double* rhs_dot, const JmgCoeffs* coeffs_dot,
                        double* phi_out, double* phi_dot_out, void* workspace, size_t workspace_bytes,
                        void* tangent_workspace, size_t tangent_workspace_bytes, jmg_stream_t stream);

/* Runs nsweeps red-black sweeps in place on the level arrays already in the workspace
 * (phi and rhs of that level as left by jmg_solve / jmg_op_*): the smoother of
 * red_black_gauss_seidel (solver_2d.py:670-692) without copies, for timing it alone. */
int jmg_op_smooth_ws(JmgPlan* plan, int level, int nsweeps, void* workspace, size_t workspace_bytes,
                     jmg_stream_t stream);
/* The same for the FP32 arrays of a mixed-precision plan (the smoother of its FP32
 * cycles), for timing it alone. */
int jmg_op_smooth32_ws(JmgPlan* plan, int level, int nsweeps, void* workspace, size_t workspace_bytes,
                       jmg_stream_t stream);

/* The coarse sub-cycle of this plan's cycles alone (the levels from
 * jmg_plan_coarse_start down to the deepest one, in one launch of the single-block
 * coarse kernel by default), on the level arrays already in the workspace: the coarse
 * branch of multigrid_cycle (solver_2d.py:582-614) without copies, for timing it alone.
 * fp32 != 0: the FP32 arrays of a mixed-precision plan. */
int jmg_op_coarse_ws(JmgPlan* plan, int fp32, void* workspace, size_t workspace_bytes, jmg_stream_t stream);
/* The exact FP64 residual that ends every step of a mixed-precision FCG solve alone
 * (rho = rhs - L_h x on level 0, its FP32 copy for the next cycle, the partial sums of
 * rho . rho), on the arrays already in the workspace, for timing it; the plan needs
 * JMG_OUTER_FCG and JMG_PREC_MIXED. No reference counterpart: the reference's stopping
 * test is a distance, and it has no Krylov outer iteration. */
int jmg_op_fcg_residual_ws(JmgPlan* plan, void* workspace, size_t workspace_bytes, jmg_stream_t stream);
/* First level the coarse sub-cycle takes (valid after the plan's first solve or
 * jmg_op_coarse_ws on a GPU; before that the single-block rule's choice). No reference
 * counterpart. */
int jmg_plan_coarse_start(const JmgPlan* plan);
/* First level of the 2D cycle that the persistent middle-level kernel takes (that level
 * and every one below it in one cooperative launch, grid barriers between the fused
 * operator pairs, the coarse sub-cycle on one of its blocks), or -1 when this plan's
 * cycles run as separate launches. Valid after the plan's first solve. No reference
 * counterpart: the middle and coarse branches of multigrid_cycle (solver_2d.py:582-614). */
int jmg_plan_mid_start(const JmgPlan* plan);

/* Whether this plan's solves run the fused operator pairs on a 2D level (fp32 != 0: the
 * FP32 cycles of a mixed plan): the last pre-sweep with the defect and restriction, the
 * prolongation with the first post-sweep, each one launch over tiles with halos. No
 * reference counterpart. */
int jmg_plan_level_fused(const JmgPlan* plan, int level, int fp32);
/* The last pre-sweep of a level followed by defect + restriction onto level + 1
 * (red_black_gauss_seidel then defect, solver_2d.py:670-692, 616-647) on the arrays
 * already in the workspace, as a solve runs them (one fused launch where
 * jmg_plan_level_fused says so), for timing them alone. No reference counterpart. */
int jmg_op_smooth_restrict_ws(JmgPlan* plan, int level, int fp32, void* workspace, size_t workspace_bytes,
                              jmg_stream_t stream);

/* Kernel launches per sweep of a level in this plan's solves (fp32 != 0: the FP32
 * cycles of a mixed plan): 1 for the one-pass 3D sweep, 2 colour passes, 4 sub-lattice
 * passes with D_xy; 0 for a bad level. No reference counterpart. */
int jmg_plan_sweep_launches(const JmgPlan* plan, int level, int fp32);

/* Kernel launches of one jmg_solve: the fixed part (copies, hierarchy, loop set-up) and
 * the part repeated per loop iteration (one cycle plus its stopping test). No reference
 * counterpart: it reports this library's launch schedule. */
int jmg_plan_launch_counts(const JmgPlan* plan, int64_t* per_solve_fixed, int64_t* per_cycle);

/* Waits for the stream and reports whether the last solve on this workspace completed its
 * device-side waits: JMG_OK, or JMG_ERR_TIMEOUT when one ran out (a grid barrier of the
 * persistent middle-level kernel, whose blocks wait on one another, or a staging copy of
 * the coarse levels). Such a wait gives up after about a second, marks the iterate with
 * NaN and ends the solve's loop, so a fault never hangs the device. No counterpart in the
 * reference, whose XLA program has no device-side waits. */
int jmg_solve_check(JmgPlan* plan, void* ws, size_t ws_bytes, jmg_stream_t stream);

/* Relative residual ||rhs - L_h phi||_2 / ||rhs||_2 over interior indices 2..m, FP64,
 * written to the device double *out, for callers that cannot allocate device memory
 * (a server that owns the whole device heap in its own pool, a plugin host that passes
 * only inputs and outputs, a loop that cannot afford an allocation's synchronisation).
 * No counterpart in the reference. It needs no plan and no workspace: its scratch is a
 * fixed 16 MiB array of this library's device memory, kept on every GPU that loads the
 * library until the process exits, so grids whose level-0 phi copy and coefficients
 * need more (roughly 2D beyond 512^2, 3D beyond 64^3) are rejected with JMG_ERR_VALUE.
 * The first call on each device looks up the array's address; make it outside stream
 * capture. All calls share the array: calls that overlap on the GPU race, so serialise
 * them. phi, rhs and the coefficient arrays are dense padded device arrays, as for
 * jmg_solve; phi's frame is read as zero, as jmg_rel_residual reads it, so the two give
 * the same number for any phi. */
int jmg_rel_residual_noalloc(const JmgGrid* grid, const double* phi, const double* rhs,
                             const JmgCoeffs* coeffs, double* out, jmg_stream_t stream);

/* ---- learned initial guess (2D) ---------------------------------------------------------
 * No counterpart in the reference, which always starts from the caller's phi0: these
 * entries predict phi0 with a small U-Net (4 levels, 16/32/64/64 channels, 3x3
 * convolutions, BF16 activations and weights, FP32 accumulation on the tensor cores) and
 * train it. The solver then iterates from that guess to the caller's tolerance, so the
 * multigrid residual judges the guess. All pointers are device pointers; x is BF16 NHWC
 * with 16 channels (16-byte aligned), y and targets are FP32 [batch][res][res]. */
typedef struct JmgNet JmgNet;
/* Number of FP32 parameters: per layer the weights [cout][3][3][cin], then the bias. */
int64_t jmg_net_num_params(void);
/* res: network resolution (a multiple of 128); max_batch: largest batch of the
 * training and gradient calls. Parameters start at zero (set them before use). */
int jmg_net_create(JmgNet** out, int res, int max_batch);
void jmg_net_destroy(JmgNet* net);
/* Copies parameters in (and resets the optimiser state) / out. */
int jmg_net_set_params(JmgNet* net, const float* params, jmg_stream_t stream);
int jmg_net_get_params(JmgNet* net, float* params, jmg_stream_t stream);
/* y = network output (channel 0) for a batch of packed inputs. */
int jmg_net_forward(JmgNet* net, const void* x, int batch, float* y, jmg_stream_t stream);
/* Mean squared error against targets: *loss (device float) and, if grads is not NULL,
 * d loss / d params (FP32, jmg_net_num_params values). */
int jmg_net_loss_grad(JmgNet* net, const void* x, const float* target, int batch, float* loss, float* grads,
                      jmg_stream_t stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on the mean squared error; the batch's
 * loss is added to *loss when loss is not NULL. */
int jmg_net_train_step(JmgNet* net, const void* x, const float* target, int batch, float lr, float* loss,
                       jmg_stream_t stream);
/* Packed network input of one square 2D problem (grid m a multiple of res): averages
 * over f x f blocks (f = m / res) of log D_xx, log D_yy, lambda / 10 and rhs, the last
 * divided by its RMS over the network grid, written to *rms_out (device float). */
int jmg_net_inputs_2d(JmgNet* net, const JmgGrid* grid, const JmgCoeffs* coeffs, const double* rhs, void* x,
                      float* rms_out, jmg_stream_t stream);
/* Training target of one problem: the block average of phi divided by out_scale * rms. */
int jmg_net_target_2d(JmgNet* net, const JmgGrid* grid, const double* phi, const float* rms, float out_scale,
                      float* target, jmg_stream_t stream);
/* phi0 (dense padded (m+3)^2 FP64) = beta * out_scale * rms * the network output,
 * bilinear from the network grid to the solver grid, zero frame; beta is the Ritz scale
 * (g . rhs) / (g . L_h g) of that field g under the level-0 operator, the factor that
 * minimises the energy-norm error (0 when it is not positive). */
int jmg_net_guess_2d(JmgNet* net, const JmgGrid* grid, const JmgCoeffs* coeffs, const double* rhs, float out_scale,
                     double* phi0, jmg_stream_t stream);

/* Message of the last failed call on this thread ("" if none). */
const char* jmg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* JMG_H */
