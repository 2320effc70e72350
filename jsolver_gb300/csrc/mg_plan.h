// mg_plan.h — the plan object behind the C ABI (internal to libjmg).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/jmg.h"
#include "mg_kernels.h"

namespace jmg {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x, size_t a = kAlign) { return (x + a - 1) / a * a; }

struct LevelInfo {
  int m[3];
  Box box;
  size_t elems;
  size_t phi, rhs, wx, wy, wz, invd, acc;   // FP64 arrays (byte offsets)
  size_t d[3];                              // 3D averaged D (levels >= 1)
  size_t phi32, rhs32, wx32, wy32, wz32, invd32, acc32;  // FP32 mirrors (mixed precision)
  size_t xd[4], xd32[4];  // 2D with D_xy: A_ll, A_rl, A_lr, A_rr (FP64, FP32 mirrors); 0 if absent
  size_t phi2, phi2_32;   // second phi buffers (FP64, FP32) of levels swept in one pass or by
                          // the fused operator pairs; 0 if absent
  bool onepass64, onepass32;  // sweeps in one pass (FP64, FP32 arrays)
  bool fuse_ops;              // grid-wide level: fused smooth + restrict, prolong + smooth
};

}  // namespace jmg

struct JmgPlan {
  JmgGrid grid;
  JmgConfig cfg;
  int dim = 2;
  int levels = 0;       // L of the reference
  int used = 0;         // levels visited: 0..L-2
  int coarse_start = 0; // first level run by one coarse sub-cycle kernel
  bool mixed = false;
  bool off_diag = false;  // 2D 9-point stencil (D_xy)
  std::vector<jmg::LevelInfo> lv;
  size_t off_phi_old = 0, off_state = 0, off_parts = 0, off_tab64 = 0, off_tab32 = 0, ws_bytes = 0;
  // outer = FCG: FP64 level-0 vectors rho (residual), d (direction), q = L d, z64 (the
  // FP64 cycle's output), three partial-sum arrays, and the FP64 level table whose level
  // 0 is (z64, rho) for the cycle that preconditions
  bool fcg = false;
  size_t off_rho = 0, off_d = 0, off_q = 0, off_z64 = 0, off_fcg_parts = 0, off_tab64z = 0;
  int nparts = 0;
  // graph cache: one executable graph per workspace address (a batched solve runs one
  // workspace per lane, each with its own graph), oldest evicted beyond kMaxGraphs
  struct GraphSlot {
    void* ws;
    cudaGraphExec_t exec;
    bool mid;  // captured with the persistent middle-level kernel
  };
  // more than the 32 lanes of a batched solve, so that a full batch alternating with
  // single solves on other workspaces keeps every lane's graph
  static constexpr int kMaxLanes = 32;
  static constexpr int kMaxGraphs = kMaxLanes + 8;
  std::vector<GraphSlot> graphs;
  cudaStream_t cap = nullptr;
  // batched solves: the lanes' streams and the events that fork them from and join them
  // to the caller's stream
  std::vector<cudaStream_t> lane_streams;
  std::vector<cudaEvent_t> lane_events;
  cudaEvent_t fork_event = nullptr;
  // reverse mode: the checkpointed forward and the reverse sweep over the cycles, captured
  // once per (workspace, adjoint workspace) address pair
  cudaGraphExec_t vjp_exec = nullptr;
  void *vjp_ws = nullptr, *vjp_aws = nullptr;
  // Host-driven loop instead of the conditional-WHILE graph (environment variable
  // JMG_HOST_LOOP=1 at plan creation): the same kernels, with the loop decision read back
  // after every iteration. Profilers cannot attribute kernel nodes inside graphs that hold
  // conditional nodes; this mode lets them see every launch.
  bool host_loop = false;
  // coarse sub-cycle on a thread-block cluster (cluster_ranks 0: the single-block
  // global-memory kernel instead, from the first level of at most 2048 points)
  int cluster_ranks = 0;
  bool coarse_ready = false;  // coarse_setup done
  bool force_block = true;    // single-block coarse kernel (JMG_COARSE=cluster at plan creation: cluster)
  jmg::ClusterLayout cluster{};
  size_t cluster_smem64 = 0, cluster_smem32 = 0;
  // FP32 2D coarse levels from shared memory (k_coarse_smem32, opt-in JMG_COARSE32=smem):
  // its dynamic shared-memory bytes, 0 when not used
  size_t coarse_smem32 = 0;
  // the single-block coarse sub-cycle with its levels staged in shared memory by bulk
  // copies (mg_coarse_staged.cu, the default): dynamic shared-memory bytes of the FP64 and
  // FP32 tables (0: the global-memory kernel instead) and the block size
  size_t coarse_staged64 = 0, coarse_staged32 = 0;
  int coarse_threads = 512;
  // 2D: the levels from mid_start down (fused operator pairs) and the coarse sub-cycle in
  // one cooperative launch (mg_mid2d.cu); mid_start -1: not used. Dynamic shared memory of
  // the FP64 and FP32 kernels (0: that precision does not use it), grid size, and the test
  // mode whose first barrier never completes (JMG_MID_STALL=1)
  int mid_start = -1;
  size_t mid_smem64 = 0, mid_smem32 = 0;
  int mid_blocks = 0;
  bool mid_stall = false;
  // whether the cycle being emitted may use it: not in the lanes of a batched solve, whose
  // concurrent cooperative launches would compete for the same SMs
  bool mid_now = false;
  bool in_batch = false;  // jmg_solve_batched is issuing its lanes' solves
};


namespace jmg {

template <typename T>
inline T* ptr(void* ws, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

// views of level l of the workspace (mg_driver.cu)
Lvl<double> lvl64(const JmgPlan* p, void* ws, int l);
Lvl<float> lvl32(const JmgPlan* p, void* ws, int l);
CycleParams cycle_params(const JmgPlan* p, bool off_diag);
// validation of a solve's coefficient arguments and workspace (mg_driver.cu)
int check_coeffs(const JmgPlan* p, const JmgCoeffs* c);
int check_ws(const JmgPlan* p, void* ws, size_t bytes);
int build_hierarchy(JmgPlan* p, const JmgCoeffs* c, void* ws, cudaStream_t s);
// chooses the coarse sub-cycle kernel once per plan (needs the GPU; mg_driver.cu)
int coarse_setup(JmgPlan* p);
// first level the single-block coarse kernel takes (at most JMG_COARSE_POINTS padded
// points, 2048 by default; mg_driver.cu)
int block_coarse_level(const JmgPlan* p);

}  // namespace jmg
