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

constexpr int kTX = 64, kTY = 8;  // interior points of a tile (x, y)
constexpr int kBX = kTX + 4;      // box width: x from i0-2 (a 16-byte aligned start)
// Boxes (rows; y from j0-2 for 12 and 11 rows, from j0-1 for 10): phi 12 (the red ring's
// neighbours), wy 11 (couplings to the row below the ring), wz, wx, rhs, 1/A_cc 10 (the
// ring's rows). Sub-box sizes are rounded up to 128 bytes.
enum { M_PHI = 0, M_WZ = 1, M_WX = 2, M_WY = 3, M_RHS = 4, M_INVD = 5, kMaps = 6 };
constexpr int kRowsPhi = 12, kRowsWy = 11, kRows10 = 10;
constexpr int kRows[kMaps] = {kRowsPhi, kRows10, kRows10, kRowsWy, kRows10, kRows10};
constexpr int kPhiE = 832, kWzE = 704;               // floats of the (phi, wz) sub-boxes
constexpr int kWxE = 704, kWyE = 768, kRhsE = 704, kInvE = 704;
constexpr int kAE = kPhiE + kWzE;                    // group A slot: phi, wz (1536 floats)
constexpr int kBE = kWxE + kWyE + kRhsE + kInvE;     // group B slot: wx, wy, rhs, invd (2880)
// Plane ring: step k issues group A of plane k+kDA and group B of plane k+kDB; group A of
// plane q is read until step q-1 and group B until step q-2, so kDA slots and kDB-1 slots
// suffice. The copies have kDA-4 and kDB-3 steps of lead beyond the step that waits for
// them.
constexpr int kDA = 4, kDB = 4;
constexpr int kASlots = kDA, kBSlots = kDB - 1;
constexpr int kRX = kTX + 2, kRY = kTY + 2;          // red ring region
constexpr int kRed = kRX * kRY / 2;                  // 330 red points per plane
constexpr int kThreads = 384;                        // black: t < 256; red: t < 330
constexpr int kBlocksPerSM = 3;
constexpr int kRedSlots = 4;
constexpr size_t kSmem = (size_t)(kASlots * kAE + kBSlots * kBE) * 4;  // 59,136 bytes
constexpr uint32_t kBytesPhi = kBX * kRowsPhi * 4, kBytesWy = kBX * kRowsWy * 4, kBytes10 = kBX * kRows10 * 4;

struct Maps {
  CUtensorMap m[kMaps];
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

// Step k of a tile's march (k from ka-3 to kb-1):
//   thread 0 issues the copies of group A of plane k+kDA and group B of plane k+kDB (into
//   the slots planes k and k+1 left);
//   the red threads compute red(k+2) from phi(k+1 .. k+3), wz(k+1 .. k+2) and the group-B
//   arrays of plane k+2;
//   the black threads (k >= ka) update black(k) from the red values in shared memory and
//   coefficients read through L2 a step ahead (their copies passed through it earlier);
//   thread 0 waits for the next step's copies; one barrier.
// Steps ka-3 .. ka-1 only produce red(ka-1), red(ka), red(ka+1).
__global__ void __launch_bounds__(kThreads, kBlocksPerSM)
    k_sweep_tma3d(const __grid_constant__ Maps maps, Lvl<float> a, float* __restrict__ out, int zero_in,
                  int per_block) {
  extern __shared__ __align__(1024) float sm[];  // [4][A slot] then [3][B slot]
  float* const sA = sm;
  float* const sB = sm + kASlots * kAE;
  __shared__ float red[kRedSlots][kRY][kRX];
  __shared__ __align__(8) uint64_t barA[kASlots], barB[kBSlots];
  const int tid = threadIdx.x;
  const int planes = a.mz - 1;  // interior planes 2 .. mz
  const int ntx = (a.mx - 1 + kTX - 1) / kTX, nty = (a.my - 1 + kTY - 1) / kTY;
  const long long total = (long long)ntx * nty * planes;
  long long g = (long long)blockIdx.x * per_block;
  const long long g1 = g + per_block < total ? g + per_block : total;
  const bool zin = zero_in != 0;
  const uint32_t bytesA = (zin ? 0u : kBytesPhi) + kBytes10;
  const uint32_t bytesB = 3 * kBytes10 + kBytesWy;
  const int P = a.P, S = (int)a.S;
  const int par = first_color_parity<3>();
  if (tid == 0) {
    for (int s = 0; s < kASlots; ++s) mbar_init(&barA[s], 1);
    for (int s = 0; s < kBSlots; ++s) mbar_init(&barB[s], 1);
  }
  pdl_enter();
  __syncthreads();
  unsigned seqA = 0, seqB = 0;        // copies of the finished segments, per group
  unsigned issuedA = 0, issuedB = 0;  // thread 0: copies issued so far
  bool ok = true;
  const bool red_role = tid < kRed;
  const int rr = red_role ? tid / (kRX / 2) : 0;
  const int rx = red_role ? 2 * (tid - rr * (kRX / 2)) : 0;
  const bool blk_role = tid < 256;
  const int tx = tid & 31, ty = tid >> 5;
  while (g < g1 && ok) {
    const int tile = (int)(g / planes);
    const int ka = 2 + (int)(g - (long long)tile * planes);
    const long long tend = (long long)(tile + 1) * planes;
    const int kb = 2 + (int)((g1 < tend ? g1 : tend) - (long long)tile * planes);  // planes ka .. kb-1
    const int i0 = 2 + kTX * (tile % ntx), j0 = 2 + kTY * (tile / ntx);
    // sequence numbers: group A plane q -> baseA + q (planes ka-2 .. kb+1), group B plane
    // q -> baseB + q (planes ka-1 .. kb)
    const unsigned baseA = seqA - (unsigned)(ka - 2), baseB = seqB - (unsigned)(ka - 1);
    const int lastA = kb + 1, lastB = kb;
    seqA = baseA + (unsigned)lastA + 1u;
    seqB = baseB + (unsigned)lastB + 1u;
    auto slotA = [&](int q) { return (baseA + (unsigned)q) % kASlots; };
    auto slotB = [&](int q) { return (baseB + (unsigned)q) % kBSlots; };
    auto issueA = [&](int q) {
      const unsigned s = slotA(q);
      float* d = sA + s * kAE;
      mbar_expect_tx(&barA[s], bytesA);
      if (!zin) tma_plane(&maps.m[M_PHI], d, i0 - 2, j0 - 2, q, &barA[s]);
      tma_plane(&maps.m[M_WZ], d + kPhiE, i0 - 2, j0 - 1, q, &barA[s]);
      ++issuedA;
    };
    auto issueB = [&](int q) {
      const unsigned s = slotB(q);
      float* d = sB + s * kBE;
      mbar_expect_tx(&barB[s], bytesB);
      tma_plane(&maps.m[M_WX], d, i0 - 2, j0 - 1, q, &barB[s]);
      tma_plane(&maps.m[M_WY], d + kWxE, i0 - 2, j0 - 2, q, &barB[s]);
      tma_plane(&maps.m[M_RHS], d + kWxE + kWyE, i0 - 2, j0 - 1, q, &barB[s]);
      tma_plane(&maps.m[M_INVD], d + kWxE + kWyE + kRhsE, i0 - 2, j0 - 1, q, &barB[s]);
      ++issuedB;
    };
    auto waitA = [&](int q) {
      const unsigned n = baseA + (unsigned)q;
      return mbar_wait(&barA[n % kASlots], (n / kASlots) & 1u, kWaitPolls);
    };
    auto waitB = [&](int q) {
      const unsigned n = baseB + (unsigned)q;
      return mbar_wait(&barB[n % kBSlots], (n / kBSlots) & 1u, kWaitPolls);
    };
    if (tid == 0) {
      for (int q = ka - 2; q <= ka + kDA - 4 && q <= lastA; ++q) issueA(q);
      for (int q = ka - 1; q <= ka + kDB - 4 && q <= lastB; ++q) issueB(q);
    }
    // red role: the ring point's elements in the 12-row and 10-row boxes (column offset 0)
    const int rj = j0 - 1 + rr;
    const bool red_row_in = red_role && rj >= 2 && rj <= a.my;
    const int e12 = (rr + 1) * kBX + (rx + 1), e10 = e12 - kBX;
    const int roff0 = par - rj - (i0 - 1) - rx;
    // black role
    const int j = j0 + ty, ie = i0 + 2 * tx;
    const int lr = ty + 1;  // ring row of j
    const bool blk_row = blk_role && j <= a.my;
    const int boff0 = par - j - ie;
    // The black update's coefficients come through L2 (about a microsecond away): they are
    // loaded one step ahead, into registers, so that their latency overlaps a whole step.
    float cz = 0.f, czm = 0.f, cy = 0.f, cym = 0.f, cx = 0.f, cxm = 0.f, crh = 0.f, cinv = 0.f;
    auto black_load = [&](int k) {
      const int ib = ie + (((boff0 - k) & 1) ^ 1);
      if (blk_row && k < kb && ib <= a.mx) {
        const int pb = k * S + j * P + ib;
        cz = __ldg(a.wz + pb), czm = __ldg(a.wz + pb - S);
        cy = __ldg(a.wy + pb), cym = __ldg(a.wy + pb - P);
        cx = __ldg(a.wx + pb), cxm = __ldg(a.wx + pb - 1);
        crh = __ldg(a.rhs + pb), cinv = __ldg(a.invd + pb);
      }
    };
    black_load(ka);
    // Thread 0 alone waits for the copies, before the barrier that ends the previous step;
    // the barrier then orders every other thread's reads after that completion. First the
    // planes of step ka-3 (red(ka-1)): phi and wz of ka-2 .. ka, the group-B arrays of ka-1.
    {
      bool miss = false;
      if (tid == 0) miss = !waitA(ka - 2) || !waitA(ka - 1) || !waitA(ka) || !waitB(ka - 1);
      if (__syncthreads_or(miss)) {
        ok = false;
        break;
      }
    }
    for (int k = ka - 3; k < kb; ++k) {
      if (tid == 0) {
        if (k + kDA <= lastA) issueA(k + kDA);
        if (k + kDB <= lastB) issueB(k + kDB);
      }
      bool miss = false;
      if (blk_row && k >= ka) {
        // black(k) from red(k-1), red(k), red(k+1); both colours of plane k out
        const float(*rm)[kRX] = red[(k - 1) & (kRedSlots - 1)];
        const float(*rc)[kRX] = red[k & (kRedSlots - 1)];
        const float(*rp)[kRX] = red[(k + 1) & (kRedSlots - 1)];
        const int roff = (boff0 - k) & 1;  // the red one of the pair: ie + roff
        const int xr = 2 * tx + 1 + roff, xb = 2 * tx + 1 + (roff ^ 1);
        const int prow = k * S + j * P;
        if (ie + roff <= a.mx) out[prow + ie + roff] = rc[lr][xr];
        const int ib = ie + (roff ^ 1);
        float v = 0.f;
        if (ib <= a.mx) {
          float s = cz * rp[lr][xb];
          s = fmaf(czm, rm[lr][xb], s);
          s = fmaf(cy, rc[lr + 1][xb], s);
          s = fmaf(cym, rc[lr - 1][xb], s);
          s = fmaf(cx, rc[lr][xb + 1], s);
          s = fmaf(cxm, rc[lr][xb - 1], s);
          s = s - crh;
          v = s * cinv;
        }
        black_load(k + 1);
        if (ib <= a.mx) out[prow + ib] = v;
      }
      if (red_role && k + 2 <= kb) {
        // red(k+2): phi(k+1 .. k+3), wz(k+1 .. k+2) and the group-B arrays of plane k+2
        {
          const int q = k + 2;
          const int off = (roff0 - q) & 1;
          const int x = rx + off;
          const int i = i0 - 1 + x;
          float v = 0.f;
          if (red_row_in && i >= 2 && i <= a.mx && q >= 2 && q <= a.mz) {
            const float* A1 = sA + slotA(q - 1) * kAE;
            const float* A2 = sA + slotA(q) * kAE;
            const float* A3 = sA + slotA(q + 1) * kAE;
            const float* B2 = sB + slotB(q) * kBE;
            const int e = e12 + off, f = e10 + off;
            const float rh = B2[kWxE + kWyE + f], inv = B2[kWxE + kWyE + kRhsE + f];
            if (zin) {
              v = (0.f - rh) * inv;
            } else {
              float s = A2[kPhiE + f] * A3[e];
              s = fmaf(A1[kPhiE + f], A1[e], s);
              s = fmaf(B2[kWxE + e], A2[e + kBX], s);
              s = fmaf(B2[kWxE + e - kBX], A2[e - kBX], s);
              s = fmaf(B2[f], A2[e + 1], s);
              s = fmaf(B2[f - 1], A2[e - 1], s);
              s = s - rh;
              v = s * inv;
            }
          }
          red[q & (kRedSlots - 1)][rr][x] = v;
        }
      }
      // the next step's planes: phi and wz of k+4, the group-B arrays of k+3
      if (tid == 0 && k + 3 <= kb) miss = !waitA(k + 4) || !waitB(k + 3);
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
      for (int s = 0; s < kASlots; ++s)
        if (issuedA > (unsigned)s) {  // the last copy issued into slot s
          const unsigned last = issuedA - 1 - ((issuedA - 1 - (unsigned)s) % kASlots);
          mbar_wait(&barA[s], (last / kASlots) & 1u, kWaitPolls);
        }
      for (int s = 0; s < kBSlots; ++s)
        if (issuedB > (unsigned)s) {
          const unsigned last = issuedB - 1 - ((issuedB - 1 - (unsigned)s) % kBSlots);
          mbar_wait(&barB[s], (last / kBSlots) & 1u, kWaitPolls);
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

// a level array (padded extents, pitched) as a 3D FP32 tensor with 68 x rows x 1 boxes
bool level_map(CUtensorMap* m, const float* base, const Lvl<float>& a, int rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)a.mx + 3, (cuuint64_t)a.my + 3, (cuuint64_t)a.mz + 3};
  const cuuint64_t strides[2] = {(cuuint64_t)a.P * 4, (cuuint64_t)a.S * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kBX, (cuuint32_t)rows, 1};
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

// the one-pass FP32 3D sweeps run here unless JMG_SWEEP3D=regs selects k_sweep_fused3d
// (read per launch, i.e. when a solve's graph is captured)
bool sweep_tma3d_enabled() {
  const char* e = getenv("JMG_SWEEP3D");
  return !(e && std::strcmp(e, "regs") == 0);
}

bool launch_sweep_tma3d(Lvl<float>& a, bool zero_in, cudaStream_t s) {
  if (!sweep_tma3d_ready()) return false;
  // the six tensor maps of a level view, encoded once and kept (a few levels and both phi
  // buffers of a solve; the host work stays out of timed loops)
  struct Entry {
    const float* src[kMaps];
    int mx, my, mz, P;
    Maps maps;
  };
  static std::mutex mu;
  static Entry cache[16];
  static int ncache = 0, next = 0;
  const float* src[kMaps] = {a.phi, a.wz, a.wx, a.wy, a.rhs, a.invd};
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
      for (int k = 0; k < kMaps; ++k)
        if (!level_map(&e.maps.m[k], src[k], a, kRows[k])) return false;
      hit = ncache < 16 ? ncache++ : next;
      if (hit == next) next = (next + 1) % 16;
      cache[hit] = e;
    }
    maps = cache[hit].maps;
  }
  // Neighbouring tiles must march up z together, so that the halo rows one block loads
  // are still in L2 when the next block loads them: every block takes an equal share of
  // one tile's plane column, as many shares per column as fill the resident blocks.
  // Ranges balanced over the blocks without regard to z read 2.1x the algorithmic bytes
  // from DRAM (ncu: L2 hit rate 17 %).
  const long long tiles = (long long)((a.mx - 1 + kTX - 1) / kTX) * ((a.my - 1 + kTY - 1) / kTY);
  const int planes = a.mz - 1;
  const long long total = tiles * planes;
  const long long resident = (long long)num_sms() * kBlocksPerSM;
  long long nchunk = tiles < resident ? resident / tiles : 1;
  if (nchunk > planes) nchunk = planes;
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
