// mg_noalloc.cu — relative residual without any device allocation by the caller.
//
// Who needs this: some callers cannot allocate device memory. An inference or
// simulation server may reserve the whole device heap up front for its own pool and
// forbid further cudaMalloc. A plugin host may hand a routine only its inputs and
// outputs, with no way to request a workspace. A hot loop may not afford the implicit
// device synchronisation a fresh allocation can cause. jmg_rel_residual needs a
// caller-provided workspace; jmg_rel_residual_noalloc computes the same number with its
// scratch in a fixed array of this library's own device memory.
//
// The scratch is a file-scope __device__ array of JMG_NOALLOC_SCRATCH_DOUBLES doubles
// (16 MiB). Every GPU that loads this library keeps it until the process exits. It
// holds a copy of phi with its frame set to zero (jmg_rel_residual copies phi into its
// workspace the same way, so a phi whose frame is not zero gives the same number in
// both; rhs is read at interior points only and needs no copy), the level-0 stencil
// coefficients (x/y(/z) face couplings, A_cc and 1/A_cc), all in the dense padded layout
// of the inputs, the per-block partial sums and the two norms. Grids whose arrays do not fit are rejected with JMG_ERR_VALUE and a message
// stating the limit.
//
// Host code cannot pass the array's name to a kernel (on the host that name is only a
// stand-in, not a device address), so the first call on each device, with that device
// current, looks up the array's device address with cudaGetSymbolAddress and caches it
// per device. Make that first call outside any stream capture.
//
// All calls share the one array and it keeps whatever the previous call left in it; the
// kernels below overwrite everything they read before reading it, so stale contents do
// not matter. Calls whose work overlaps on the GPU (on different streams, or different
// host threads on the same device) race on the array: serialise them.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/jmg.h"
#include "mg_kernels.h"

using namespace jmg;

#define JMG_NOALLOC_SCRATCH_DOUBLES (2u * 1024u * 1024u)
#define JMG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[JMG_NOALLOC_SCRATCH_DOUBLES];

namespace {

std::mutex g_noalloc_mutex;
double* g_scratch_addr[JMG_NOALLOC_MAX_DEVICES] = {nullptr};

// the message is reported by jmg_last_error(), like every other failure
int noalloc_err(int code, const std::string& msg) { return jmg::set_error_message(code, msg.c_str()); }

// Device address of the scratch array on the current device (looked up once per device).
int scratch_for_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_err(JMG_ERR_CUDA, std::string("cudaGetDevice failed: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= JMG_NOALLOC_MAX_DEVICES) return noalloc_err(JMG_ERR_CUDA, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return noalloc_err(JMG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return JMG_OK;
}

}  // namespace

extern "C" {

// Relative residual ||rhs - L_h phi||_2 / ||rhs||_2 over the interior indices 2..m of
// level 0, in FP64, written to the device double *out. Same kernels and the same number
// as jmg_rel_residual (phi's frame is read as zero in both), without a workspace. See the
// file header for the scratch rules.
int jmg_rel_residual_noalloc(const JmgGrid* grid, const double* phi, const double* rhs, const JmgCoeffs* coeffs,
                             double* out, jmg_stream_t stream) {
  if (!grid || !phi || !rhs || !coeffs || !out) return noalloc_err(JMG_ERR_VALUE, "NULL argument");
  const int dim = grid->ndim;
  if (dim != 2 && dim != 3) return noalloc_err(JMG_ERR_VALUE, "ndim must be 2 or 3");
  for (int a = 0; a < dim; ++a)
    if (grid->m[a] < 2) return noalloc_err(JMG_ERR_VALUE, "each resolution must be at least 2");
  int nscalar = 0;
  for (int a = 0; a < dim; ++a)
    if (coeffs->D[a] == nullptr) ++nscalar;
  if (nscalar != 0 && nscalar != dim)
    return noalloc_err(JMG_ERR_VALUE, "Shape mismatch: the D components must be all scalars or all arrays.");
  if (coeffs->D_xy && dim == 3) return noalloc_err(JMG_ERR_VALUE, "D_xy is a 2D argument");
  if (coeffs->D_xy && nscalar == 0)
    return noalloc_err(JMG_ERR_VALUE, "jmg_rel_residual_noalloc takes no D_xy: its fixed scratch holds the "
                                      "5-point coefficients only; use jmg_rel_residual");

  // dense padded layout of the caller's arrays
  Box b;
  b.nx = grid->m[0] + 3;
  b.ny = grid->m[1] + 3;
  b.nz = dim == 3 ? grid->m[2] + 3 : 1;
  b.P = b.nx;
  b.S = (long long)b.nx * b.ny;
  const unsigned long long n = (unsigned long long)b.S * b.nz;
  const unsigned long long n_al = (n + 31) / 32 * 32;  // keep every array 256-byte aligned
  const int nparts = residual_num_parts(dim, b);
  const unsigned long long state_doubles = (sizeof(LoopState) + 255) / 256 * 32;
  // phi with a zero frame, dim face arrays, A_cc, 1/A_cc; partial sums; loop state
  const unsigned long long need = (unsigned long long)(dim + 3) * n_al + (unsigned long long)(nparts + 31) / 32 * 32 +
                                  state_doubles;
  if (need > JMG_NOALLOC_SCRATCH_DOUBLES) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "grid too large for jmg_rel_residual_noalloc: needs %llu doubles of scratch, the fixed limit is %u "
             "(16 MiB); use jmg_rel_residual with a workspace",
             need, JMG_NOALLOC_SCRATCH_DOUBLES);
    return noalloc_err(JMG_ERR_VALUE, msg);
  }
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != JMG_OK) return rc;

  Lvl<double> a{};
  a.phi = scratch;
  a.rhs = const_cast<double*>(rhs);  // read at interior points only
  a.wx = scratch + n_al;
  a.wy = scratch + 2 * n_al;
  a.wz = dim == 3 ? scratch + 3 * n_al : nullptr;
  a.acc = scratch + (dim == 3 ? 4 : 3) * n_al;
  a.invd = a.acc + n_al;
  double* parts = a.invd + n_al;
  LoopState* st = reinterpret_cast<LoopState*>(parts + (nparts + 31) / 32 * 32);
  a.mx = grid->m[0];
  a.my = grid->m[1];
  a.mz = dim == 3 ? grid->m[2] : 0;
  a.P = b.P;
  a.S = b.S;

  HierInputs in;
  in.lam = coeffs->lam;
  in.lam_scalar = coeffs->lam_scalar;
  in.scalar_lam = coeffs->lam == nullptr;
  for (int k = 0; k < 3; ++k) {
    in.D[k] = k < dim ? coeffs->D[k] : nullptr;
    in.D_scalar[k] = k < dim ? coeffs->D_scalar[k] : 0.0;
  }
  in.scalar_D = nscalar == dim;
  double sq[3] = {0, 0, 0}, idl[3] = {0, 0, 0};
  for (int k = 0; k < dim; ++k) {
    idl[k] = grid->idel[k];
    sq[k] = grid->idel[k] * grid->idel[k];
  }

  cudaStream_t s = (cudaStream_t)stream;
  // phi with a zero frame, as jmg_rel_residual copies it (the defect at i = 2 and i = m
  // reads phi at the frame indices 1 and m + 1)
  launch_copy_in(b, phi, a.phi, 1, s);
  // level-0 coefficients over the whole box (every scratch value read below is written here)
  launch_hierarchy_level(dim, 0, a, b, b, in, idl, sq, nullptr, nullptr, b, s);
  launch_residual_partials<double>(dim, a, nullptr, parts, nparts, s);
  launch_rhs_norm(st, parts, nparts, s);
  launch_residual_partials<double>(dim, a, a.phi, parts, nparts, s);
  launch_rel_residual_out(st, parts, nparts, out, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_err(JMG_ERR_CUDA, std::string("launch failed: ") + cudaGetErrorString(e));
  return JMG_OK;
}

}  // extern "C"
