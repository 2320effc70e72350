// mg_dual.cuh — dual numbers (value, tangent) for the forward-mode solve.
//
// The reference gets forward-mode derivatives by jax.jvp through its solve, fixed loop
// or dynamic while_loop alike (solver_2d.py:461-477; tests/test_solver_2d.py:173-176,
// tests/test_solver_3d.py:208-211). Here a Dual carries a value and its tangent through
// the very kernels of the solver (colour sweeps, grid restriction, cell prolongation,
// the single-block coarse cycle), which are templates over the element type. The value
// part of every operation is the FP64 operation of the plain solver (the same fma, the
// same order), so the primal iterate is bit-identical to jmg_solve's and a dynamic loop
// stops after the same number of cycles; the tangent part is the product rule:
//   (a * b)'      = a' b + a b'
//   fma(a, b, c)' = a' b + a b' + c'
// Division does not occur: the solver multiplies by 1/A_cc, whose tangent
// -(1/A_cc)^2 A_cc' is built with the coefficient hierarchy (mg_tangent.cu).
#pragma once
#include <cuda_runtime.h>

namespace jmg {
// In a namespace of its own: the Dual overload of fma is found by argument-dependent
// lookup for Dual operands only, so unqualified fma on doubles in namespace jmg still
// names CUDA's fma.
namespace dualnum {

struct __align__(16) Dual {
  double v;  // value
  double d;  // tangent
  Dual() = default;
  __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}
  __host__ __device__ constexpr Dual(double x, double t) : v(x), d(t) {}
};

__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, ::fma(a.d, b.v, a.v * b.d)); }
__device__ __forceinline__ Dual fma(Dual a, Dual b, Dual c) {
  return Dual(::fma(a.v, b.v, c.v), ::fma(a.d, b.v, ::fma(a.v, b.d, c.d)));
}

}  // namespace dualnum
using dualnum::Dual;
}  // namespace jmg
