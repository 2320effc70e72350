// mg_fusedops2d.cu — the grid-wide kernels of the 2D fused operator pairs: one tile per
// block (the tile bodies and their description are in mg_fusedops2d.cuh).
#include "mg_common.cuh"
#include "mg_fusedops2d.cuh"
#include "mg_kernels.h"

namespace jmg {

namespace {

template <typename T, int CJ, int CI, int NT>
__global__ void __launch_bounds__(NT) k_smooth_restrict2d(Lvl<T> f, T* __restrict__ out, Lvl<T> c, int zero_in) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smraw[];
  smooth_restrict_tile<T, CJ, CI, NT, false>(f, out, c, zero_in, blockIdx.y, blockIdx.x, smraw);
}

// FP32: held to 32 registers, so 4 blocks of 512 threads fit on an SM and the 512 tiles of
// a 1024^2 level run in one wave (608 resident blocks; at 34 registers 3 fitted, 456)
template <typename T, int TJ, int TI, int NT>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 4 : 0) k_prolong_smooth2d(Lvl<T> f, T* __restrict__ out, Lvl<T> c) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smraw[];
  prolong_smooth_tile<T, TJ, TI, NT, false>(f, out, c, blockIdx.y, blockIdx.x, smraw);
}

template <typename T>
bool set_smem_attrs() {
  using F = FusedShape<T>;
  static const bool ok = [] {
    const int a = (int)SR<T, F::CJ, F::CI>::smem, b = (int)PS<T, F::TJ, F::TI>::smem;
    return cudaFuncSetAttribute(k_smooth_restrict2d<T, F::CJ, F::CI, F::NT_SR>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, a) == cudaSuccess &&
           cudaFuncSetAttribute(k_prolong_smooth2d<T, F::TJ, F::TI, F::NT_PS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess;
  }();
  return ok;
}

}  // namespace

template <typename T>
void launch_smooth_restrict2d(Lvl<T>& f, const Lvl<T>& c, bool zero_in, cudaStream_t s) {
  using F = FusedShape<T>;
  set_smem_attrs<T>();
  dim3 g((unsigned)((c.mx + 3 + F::CI - 1) / F::CI), (unsigned)((c.my + 3 + F::CJ - 1) / F::CJ));
  launch_k(k_smooth_restrict2d<T, F::CJ, F::CI, F::NT_SR>, g, dim3(F::NT_SR), SR<T, F::CJ, F::CI>::smem, s, f,
           f.phi2, c, zero_in ? 1 : 0);
  T* t = f.phi;
  f.phi = f.phi2;
  f.phi2 = t;
}

template <typename T>
void launch_prolong_smooth2d(Lvl<T>& f, const Lvl<T>& c, cudaStream_t s) {
  using F = FusedShape<T>;
  set_smem_attrs<T>();
  dim3 g((unsigned)((f.mx - 1 + F::TI - 1) / F::TI), (unsigned)((f.my - 1 + F::TJ - 1) / F::TJ));
  launch_k(k_prolong_smooth2d<T, F::TJ, F::TI, F::NT_PS>, g, dim3(F::NT_PS), PS<T, F::TJ, F::TI>::smem, s, f,
           f.phi2, c);
  T* t = f.phi;
  f.phi = f.phi2;
  f.phi2 = t;
}

void prepare_fused_ops2d() {
  set_smem_attrs<float>();
  set_smem_attrs<double>();
}

template void launch_smooth_restrict2d<float>(Lvl<float>&, const Lvl<float>&, bool, cudaStream_t);
template void launch_smooth_restrict2d<double>(Lvl<double>&, const Lvl<double>&, bool, cudaStream_t);
template void launch_prolong_smooth2d<float>(Lvl<float>&, const Lvl<float>&, cudaStream_t);
template void launch_prolong_smooth2d<double>(Lvl<double>&, const Lvl<double>&, cudaStream_t);

}  // namespace jmg
