// mg_batch.cu — many independent solves of one plan in one call.
//
// The reference's use in variational inference solves many problems of one grid
// (jax.vmap over solve_2d / solve_3d; README.md:107, examples/benchmark.py:1109-1230).
// Small grids leave most of the GPU idle in one solve: each level's kernels cover a few
// thousand points and the coarse levels run in one block. Here the problems are spread
// over lanes: every lane owns a slice of the workspace, a stream and (through the plan's
// graph cache, keyed by workspace address) its own captured solve graph, and runs its
// problems one after another while the lanes run side by side. Events fork the lanes from
// the caller's stream and join them back, so the call is ordered like one kernel launch on
// that stream. Every problem runs exactly the kernels of jmg_solve on its own workspace,
// so its result and count are those of a single solve.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/jmg.h"
#include "mg_plan.h"

namespace jmg {
int set_error_message(int code, const char* msg);
}

using namespace jmg;

namespace {

constexpr int kMaxLanes = JmgPlan::kMaxLanes;

size_t lane_bytes(const JmgPlan* p) { return align_up(p->ws_bytes); }

int fail(int code, const char* msg) { return set_error_message(code, msg); }

int ensure_lanes(JmgPlan* p, int lanes) {
  if (!p->fork_event && cudaEventCreateWithFlags(&p->fork_event, cudaEventDisableTiming) != cudaSuccess)
    return fail(JMG_ERR_CUDA, "cudaEventCreate failed");
  while ((int)p->lane_streams.size() < lanes) {
    cudaStream_t s = nullptr;
    cudaEvent_t e = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      return fail(JMG_ERR_CUDA, "cudaStreamCreate failed");
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaStreamDestroy(s);
      return fail(JMG_ERR_CUDA, "cudaEventCreate failed");
    }
    p->lane_streams.push_back(s);
    p->lane_events.push_back(e);
  }
  return JMG_OK;
}

const double* at(const double* base, int64_t stride, int b) { return base ? base + stride * b : nullptr; }

}  // namespace

extern "C" {

size_t jmg_batched_workspace_bytes(const JmgPlan* p, int32_t lanes) {
  if (!p || lanes < 1) return 0;
  return lane_bytes(p) * (size_t)std::min(lanes, (int32_t)kMaxLanes);
}

int jmg_solve_batched(JmgPlan* p, int32_t batch, const double* phi0, const double* rhs, const JmgCoeffs* c,
                      const JmgBatchStrides* strides, double* phi_out, int64_t* counts_out, void* ws,
                      size_t ws_bytes, jmg_stream_t stream) {
  if (!p) return fail(JMG_ERR_VALUE, "NULL plan");
  if (batch < 0) return fail(JMG_ERR_VALUE, "batch must be >= 0");
  if (!c || !strides) return fail(JMG_ERR_VALUE, "NULL argument");
  if (batch == 0) return JMG_OK;
  if (!phi0 || !rhs || !phi_out) return fail(JMG_ERR_VALUE, "phi0, rhs and phi_out must not be NULL");
  const size_t lb = lane_bytes(p);
  if (!ws || reinterpret_cast<uintptr_t>(ws) % kAlign) return fail(JMG_ERR_WORKSPACE, "workspace missing or misaligned");
  const int lanes = (int)std::min<size_t>({(size_t)batch, ws_bytes / lb, (size_t)kMaxLanes});
  if (lanes < 1) return fail(JMG_ERR_WORKSPACE, "workspace smaller than one lane (jmg_batched_workspace_bytes(plan, 1))");
  for (int a = 0; a < 3; ++a)
    if (strides->D[a] < 0) return fail(JMG_ERR_VALUE, "strides must be >= 0");
  if (strides->lam < 0 || strides->D_xy < 0) return fail(JMG_ERR_VALUE, "strides must be >= 0");
  int rc = ensure_lanes(p, lanes);
  if (rc) return rc;
  const Box b0 = p->lv[0].box;
  const int64_t n = (int64_t)b0.nx * b0.ny * b0.nz;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaEventRecord(p->fork_event, s) != cudaSuccess) return fail(JMG_ERR_CUDA, "cudaEventRecord failed");
  for (int l = 0; l < lanes; ++l)
    if (cudaStreamWaitEvent(p->lane_streams[l], p->fork_event, 0) != cudaSuccess)
      return fail(JMG_ERR_CUDA, "cudaStreamWaitEvent failed");
  // problems in lane order; the first error stops issuing, the lanes are joined either way
  p->in_batch = true;
  for (int b = 0; b < batch && rc == JMG_OK; ++b) {
    const int l = b % lanes;
    JmgCoeffs cb = *c;
    cb.lam = at(c->lam, strides->lam, b);
    for (int a = 0; a < 3; ++a) cb.D[a] = at(c->D[a], strides->D[a], b);
    cb.D_xy = at(c->D_xy, strides->D_xy, b);
    rc = jmg_solve(p, phi0 + n * b, rhs + n * b, &cb, phi_out + n * b, counts_out ? counts_out + b : nullptr,
                   static_cast<char*>(ws) + lb * l, lb, p->lane_streams[l]);
  }
  p->in_batch = false;
  for (int l = 0; l < lanes; ++l) {
    const bool ok = cudaEventRecord(p->lane_events[l], p->lane_streams[l]) == cudaSuccess &&
                    cudaStreamWaitEvent(s, p->lane_events[l], 0) == cudaSuccess;
    if (!ok && rc == JMG_OK) rc = fail(JMG_ERR_CUDA, "joining the lanes failed");
  }
  return rc;
}

}  // extern "C"
