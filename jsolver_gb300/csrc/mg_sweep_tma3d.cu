// mg_sweep_tma3d.cu — the one-pass 3D red-black sweep of FP32 levels with its plane tiles
// fed by the tensor-memory accelerator (cp.async.bulk.tensor) through an mbarrier ring.
//
// The same march as k_sweep_fused3d (mg_fused.cu): a block owns 64 x 8 interior columns
// and walks up z, keeping the new red values of four planes in shared memory; step k
// updates black(k) from red(k-1), red(k), red(k+1), writes both colours of plane k and
// computes red(k+2). Here every input comes from shared memory: for each plane q the six
// arrays phi (old), rhs, wx, wy, wz and 1/A_cc arrive as one 68 x 12 box each (the tile,
// a two-point ring for the red ring's neighbours) by six TMA copies that complete on the
// plane's mbarrier. Eight plane slots form a ring: step k uses planes k-1 .. k+3 and the
// copies of planes k+4 .. k+6 are in flight, so about three planes of DRAM traffic per SM
// overlap the arithmetic, and no thread computes a load address. Out-of-range boxes are
// zero-filled by the copy engine (the frame of phi is zero as well).
//
// Work: a block walks a contiguous range of the (tile, plane) list, tile-major: a whole
// plane column of its tile on large levels, so that neighbouring tiles climb together and
// share their halo rows through L2; on small levels columns are cut into chunks to fill
// the SMs, and a range that crosses into the next tile restarts the march there (three
// red planes of prologue).
//
// Every value is gs_point3d's arithmetic in the same order, so the result is
// bit-identical to the colour passes and to k_sweep_fused3d (solver_3d.py:679-706).
// Every wait on an mbarrier is bounded; one that runs out sets the table fault flag and
// fills the output with NaN (then waits, bounded, for the copies in flight).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "mg_bulk.cuh"
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

constexpr int kTX = 64, kTY = 8;           // interior points of a tile (x, y)
constexpr int kBX = kTX + 4, kBY = kTY + 4; // box: x from i0-2, y from j0-2
constexpr int kBoxBytes = kBX * kBY * 4;    // 3264
constexpr int kSlotElems = 832;             // 3328 bytes: boxes start on 128-byte boundaries
constexpr int kArrays = 6;                  // phi, rhs, wx, wy, wz, invd
enum { A_PHI = 0, A_RHS = 1, A_WX = 2, A_WY = 3, A_WZ = 4, A_INVD = 5 };
constexpr int kSlots = 8;                   // plane ring
constexpr int kAhead = 3;                   // planes in flight beyond the step's window
constexpr int kRX = kTX + 2, kRY = kTY + 2; // red ring region
constexpr int kRed = kRX * kRY / 2;         // 330 red points per plane
constexpr int kBlack = 256;                // black role: 8 warps, two points per thread
constexpr int kThreads = 640;               // + 330 red-role threads (11 warps) and spare lanes
constexpr int kRedSlots = 4;
constexpr size_t kSmem = (size_t)kSlots * kArrays * kSlotElems * 4;  // 159,744 bytes

struct Maps {
  CUtensorMap m[kArrays];
};

__device__ __forceinline__ void tma_plane(const CUtensorMap* map, float* dst, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// set by a block whose wait for its copies ran out (read and cleared by jmg_solve_check)
__device__ int g_tma_fault;

__global__ void __launch_bounds__(kThreads, 1)
    k_sweep_tma3d(const __grid_constant__ Maps maps, Lvl<float> a, float* __restrict__ out, int zero_in,
                  int per_block) {
  extern __shared__ __align__(1024) float ring[];  // [slot][array][12][68] (832-float pitch)
  __shared__ float red[kRedSlots][kRY][kRX];
  __shared__ __align__(8) uint64_t bar[kSlots];
  const int tid = threadIdx.x;
  const int planes = a.mz - 1;  // interior planes 2 .. mz
  const int ntx = (a.mx - 1 + kTX - 1) / kTX, nty = (a.my - 1 + kTY - 1) / kTY;
  const long long total = (long long)ntx * nty * planes;
  long long g = (long long)blockIdx.x * per_block;
  const long long g1 = g + per_block < total ? g + per_block : total;
  const bool zin = zero_in != 0;
  const int first = zin ? 1 : 0;  // phi is not copied from a zero initial guess
  const uint32_t bytes = (uint32_t)((kArrays - first) * kBoxBytes);
  const int P = a.P, S = (int)a.S;
  const int par = first_color_parity<3>();
  if (tid == 0)
    for (int s = 0; s < kSlots; ++s) mbar_init(&bar[s], 1);
  pdl_enter();
  __syncthreads();
  unsigned seq = 0;     // planes of the finished segments (slot = seq % 8, phase = seq / 8)
  unsigned issued = 0;  // thread 0: planes issued so far
  bool ok = true;
  // Roles in separate warps, so that a step's black and red updates run side by side:
  // black, warps 0-7: tile row ty, columns 2tx, 2tx+1 (thread 0 also issues the copies);
  // red, threads 256 .. 585: one point of the ring region per plane (row rr, pair rx).
  const bool blk_role = tid < kBlack;
  const int tx = tid & 31, ty = tid >> 5;
  const int rt = tid - kBlack;
  const bool red_role = rt >= 0 && rt < kRed;
  const int rr = red_role ? rt / (kRX / 2) : 0;
  const int rx = red_role ? 2 * (rt - rr * (kRX / 2)) : 0;
  while (g < g1 && ok) {
    const int tile = (int)(g / planes);
    const int ka = 2 + (int)(g - (long long)tile * planes);
    const long long tend = (long long)(tile + 1) * planes;
    const int kb = 2 + (int)((g1 < tend ? g1 : tend) - (long long)tile * planes);  // planes ka .. kb-1
    const int i0 = 2 + kTX * (tile % ntx), j0 = 2 + kTY * (tile / ntx);
    const unsigned base = seq - (unsigned)(ka - 2);  // sequence number of plane q: base + q
    const int last_issue = kb + 1;                   // red(kb) reads phi(kb + 1)
    seq = base + (unsigned)last_issue + 1u;
    if (tid == 0)
      for (int q = ka - 2; q <= ka + kSlots - 3 && q <= last_issue; ++q) {
        const unsigned sl = (base + (unsigned)q) & (kSlots - 1);
        mbar_expect_tx(&bar[sl], bytes);
        for (int arr = first; arr < kArrays; ++arr)
          tma_plane(&maps.m[arr], ring + (sl * kArrays + arr) * kSlotElems, i0 - 2, j0 - 2, q, &bar[sl]);
        ++issued;
      }
    auto plane = [&](int q) -> const float* { return ring + ((base + (unsigned)q) & (kSlots - 1)) * (kArrays * kSlotElems); };
    auto wait = [&](int q) {
      const unsigned n = base + (unsigned)q;
      return mbar_wait(&bar[n & (kSlots - 1)], (n >> 3) & 1u, kWaitPolls);
    };
    // red role: its ring point's box element for column offset 0, and whether the row is
    // interior; the red one of the pair alternates with the plane
    const int rj = j0 - 1 + rr;
    const bool red_row_in = red_role && rj >= 2 && rj <= a.my;
    const int e0 = (rr + 1) * kBX + (rx + 1);
    const int roff0 = par - rj - (i0 - 1) - rx;
    auto red_value = [&](int q, int* xs) -> float {
      const int off = (roff0 - q) & 1;
      *xs = rx + off;
      const int i = i0 - 1 + rx + off;
      if (!(red_row_in && i >= 2 && i <= a.mx && q >= 2 && q <= a.mz)) return 0.f;
      const int e = e0 + off;
      const float* p1 = plane(q - 1);
      const float* p2 = plane(q);
      const float rh = p2[A_RHS * kSlotElems + e], inv = p2[A_INVD * kSlotElems + e];
      if (zin) return (0.f - rh) * inv;
      const float* p3 = plane(q + 1);
      const float* ph = p2 + A_PHI * kSlotElems;
      float s = p2[A_WZ * kSlotElems + e] * p3[A_PHI * kSlotElems + e];
      s = fmaf(p1[A_WZ * kSlotElems + e], p1[A_PHI * kSlotElems + e], s);
      s = fmaf(p2[A_WY * kSlotElems + e], ph[e + kBX], s);
      s = fmaf(p2[A_WY * kSlotElems + e - kBX], ph[e - kBX], s);
      s = fmaf(p2[A_WX * kSlotElems + e], ph[e + 1], s);
      s = fmaf(p2[A_WX * kSlotElems + e - 1], ph[e - 1], s);
      s = s - rh;
      return s * inv;
    };
    // prologue: planes ka-2 .. ka+2 present, red(ka-1), red(ka), red(ka+1)
    bool bad = false;
    for (int q = ka - 2; q <= ka + 2; ++q) bad = bad || !wait(q);
    if (__syncthreads_or(bad)) {
      ok = false;
      break;
    }
    if (red_role)
      for (int q = ka - 1; q <= ka + 1; ++q) {
        int x;
        const float v = red_value(q, &x);
        red[q & (kRedSlots - 1)][rr][x] = v;
      }
    __syncthreads();
    const int j = j0 + ty, ie = i0 + 2 * tx;
    const int lr = ty + 1;                         // ring row of j
    const int eb = (ty + 2) * kBX + (2 * tx + 2);  // box element of (ie, j)
    const bool blk_row = blk_role && j <= a.my;
    const int boff0 = par - j - ie;
    for (int k = ka; k < kb; ++k) {
      if (tid == 0 && k + kAhead + 3 <= last_issue) {
        // the copies of plane k+6 into the slot plane k-2 left (its last reader was step k-1)
        const int q = k + kAhead + 3;
        const unsigned sl = (base + (unsigned)q) & (kSlots - 1);
        mbar_expect_tx(&bar[sl], bytes);
        for (int arr = first; arr < kArrays; ++arr)
          tma_plane(&maps.m[arr], ring + (sl * kArrays + arr) * kSlotElems, i0 - 2, j0 - 2, q, &bar[sl]);
        ++issued;
      }
      bool miss = false;
      if (blk_row) {
        // black(k) from red(k-1), red(k), red(k+1); both colours of plane k out. Plane k
        // completed long ago (it is waited on here only to observe that completion).
        miss = !wait(k);
        const float(*rm)[kRX] = red[(k - 1) & (kRedSlots - 1)];
        const float(*rc)[kRX] = red[k & (kRedSlots - 1)];
        const float(*rp)[kRX] = red[(k + 1) & (kRedSlots - 1)];
        const int roff = (boff0 - k) & 1;  // the red one of the pair: ie + roff
        const int xr = 2 * tx + 1 + roff, xb = 2 * tx + 1 + (roff ^ 1);
        const long long prow = (long long)k * S + (long long)j * P;
        if (ie + roff <= a.mx) out[prow + ie + roff] = rc[lr][xr];
        const int ib = ie + (roff ^ 1);
        if (ib <= a.mx && !miss) {
          const int e = eb + (roff ^ 1);
          const float* b0 = plane(k);
          const float* bm = plane(k - 1);
          float s = b0[A_WZ * kSlotElems + e] * rp[lr][xb];
          s = fmaf(bm[A_WZ * kSlotElems + e], rm[lr][xb], s);
          s = fmaf(b0[A_WY * kSlotElems + e], rc[lr + 1][xb], s);
          s = fmaf(b0[A_WY * kSlotElems + e - kBX], rc[lr - 1][xb], s);
          s = fmaf(b0[A_WX * kSlotElems + e], rc[lr][xb + 1], s);
          s = fmaf(b0[A_WX * kSlotElems + e - 1], rc[lr][xb - 1], s);
          s = s - b0[A_RHS * kSlotElems + e];
          out[prow + ib] = s * b0[A_INVD * kSlotElems + e];
        }
      } else if (red_role && k + 2 <= kb) {
        // red(k+2) (needs plane k+3) into the red slot black(k-1) read last step
        miss = !wait(k + 3);
        if (!miss) {
          int x;
          const float v = red_value(k + 2, &x);
          red[(k + 2) & (kRedSlots - 1)][rr][x] = v;
        }
      }
      if (__syncthreads_or(miss)) {
        ok = false;
        break;
      }
    }
    g = (long long)(tile + 1) * planes;
    if (g > g1) g = g1;
  }
  if (!ok) {
    // a copy did not arrive: the sweep's output is void; mark it, then (thread 0) wait,
    // bounded, for the copies still in flight before the block's shared memory goes away
    const long long n = (long long)a.S * (a.mz + 3);
    for (long long e = (long long)blockIdx.x * kThreads + tid; e < n; e += (long long)gridDim.x * kThreads)
      out[e] = __int_as_float(0x7fc00000);
    if (tid == 0) {
      atomicExch(&g_tma_fault, 1);
      for (int s = 0; s < kSlots; ++s)
        if (issued > (unsigned)s) {  // the last plane issued into slot s
          const unsigned last = issued - 1 - ((issued - 1 - (unsigned)s) & (kSlots - 1));
          mbar_wait(&bar[s], (last >> 3) & 1u, kWaitPolls);
        }
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// a level array (padded extents, pitched) as a 3D FP32 tensor with 68 x 12 x 1 boxes
bool level_map(CUtensorMap* m, const float* base, const Lvl<float>& a) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)a.mx + 3, (cuuint64_t)a.my + 3, (cuuint64_t)a.mz + 3};
  const cuuint64_t strides[2] = {(cuuint64_t)a.P * 4, (cuuint64_t)a.S * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kBX, (cuuint32_t)kBY, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      v = 0;
    return v;
  }();
  return n;
}

}  // namespace

// Whether the TMA sweep can run (encoder present, shared memory granted); checked once.
bool sweep_tma3d_ready() {
  static const bool ok = [] {
    if (!encoder() || num_sms() < 1) return false;
    return cudaFuncSetAttribute(k_sweep_tma3d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem) ==
           cudaSuccess;
  }();
  return ok;
}

// Reads (and clears) the flag of a TMA sweep whose copies did not arrive.
int sweep_tma3d_fault() {
  int v = 0;
  if (!sweep_tma3d_ready()) return 0;
  if (cudaMemcpyFromSymbol(&v, g_tma_fault, sizeof(int)) != cudaSuccess) return 0;
  if (v) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_tma_fault, &zero, sizeof(int));
  }
  return v;
}

// JMG_SWEEP3D=tma selects this kernel for the one-pass FP32 3D sweeps (read per launch,
// i.e. when a solve's graph is captured); k_sweep_fused3d stays the default
bool sweep_tma3d_enabled() {
  const char* e = getenv("JMG_SWEEP3D");
  return e && std::strcmp(e, "tma") == 0;
}

bool launch_sweep_tma3d(Lvl<float>& a, bool zero_in, cudaStream_t s) {
  if (!sweep_tma3d_ready()) return false;
  // the six tensor maps of a level view, encoded once and kept (a few levels and both phi
  // buffers of a solve; the host work stays out of timed loops)
  struct Entry {
    const float* src[kArrays];
    int mx, my, mz, P;
    Maps maps;
  };
  static std::mutex mu;
  static Entry cache[16];
  static int ncache = 0, next = 0;
  const float* src[kArrays] = {a.phi, a.rhs, a.wx, a.wy, a.wz, a.invd};
  Maps maps;
  {
    std::lock_guard<std::mutex> lock(mu);
    int hit = -1;
    for (int c = 0; c < ncache && hit < 0; ++c) {
      const Entry& e = cache[c];
      if (e.mx == a.mx && e.my == a.my && e.mz == a.mz && e.P == a.P && !std::memcmp(e.src, src, sizeof(src))) hit = c;
    }
    if (hit < 0) {
      Entry e;
      std::memset(&e, 0, sizeof(e));
      std::memcpy(e.src, src, sizeof(src));
      e.mx = a.mx, e.my = a.my, e.mz = a.mz, e.P = a.P;
      for (int k = 0; k < kArrays; ++k)
        if (!level_map(&e.maps.m[k], src[k], a)) return false;
      hit = ncache < 16 ? ncache++ : next;
      if (hit == next) next = (next + 1) % 16;
      cache[hit] = e;
    }
    maps = cache[hit].maps;
  }
  // Neighbouring tiles must march up z together, so that the halo rows one block loads
  // are still in L2 when the next block loads them: every block takes whole plane columns
  // (chunks of one when there are fewer tiles than SMs). Ranges balanced over the SMs
  // without regard to z read 2.1x the algorithmic bytes from DRAM (ncu: L2 hit rate 17 %).
  const long long tiles = (long long)((a.mx - 1 + kTX - 1) / kTX) * ((a.my - 1 + kTY - 1) / kTY);
  const int planes = a.mz - 1;
  const long long total = tiles * planes;
  const long long nchunk = tiles < num_sms() ? num_sms() / tiles : 1;
  const int per_block = (int)((planes + nchunk - 1) / nchunk);
  const int blocks = (int)((total + per_block - 1) / per_block);
  launch_k(k_sweep_tma3d, dim3((unsigned)blocks), dim3(kThreads), kSmem, s, maps, a, a.phi2, zero_in ? 1 : 0,
           per_block);
  float* t = a.phi;
  a.phi = a.phi2;
  a.phi2 = t;
  return true;
}

}  // namespace jmg
