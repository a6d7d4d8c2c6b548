// Shared definitions of the GB300 explicit-dynamics engine: the hex8 element's
// corner/integration-point numbering, launch helpers and device layouts.
//
// Numbering (reference src/nimble_element.cc:55-171): corner c and integration
// point c share the sign triple kSign[c] = (sx, sy, sz); corner c sits at
// natural coordinates kSign[c], integration point c at kSign[c] * g with
// g = 0.577350269189626 (the reference's literal, :58), all weights 1.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nsm {

// Material models (the reference's MaterialFactory names,
// src/nimble_material_factory.cc:57-70).
constexpr int kNeohookean = 0;  // "neohookean", src/nimble_material.cc:252-310
constexpr int kElastic    = 1;  // "elastic", src/nimble_material.cc:98-126
constexpr int kExternal   = 2;  // computed by a registered block-material callback (the plugin path)

// Natural coordinate of the Gauss points (src/nimble_element.cc:58).
constexpr double kGauss = 0.577350269189626;

// Sign bits of corner / integration point c: bit set = "+" side.
__host__ __device__ constexpr int sx_of(int c) { return (c == 1 || c == 2 || c == 5 || c == 6) ? 1 : 0; }
__host__ __device__ constexpr int sy_of(int c) { return (c == 2 || c == 3 || c == 6 || c == 7) ? 1 : 0; }
__host__ __device__ constexpr int sz_of(int c) { return c >= 4 ? 1 : 0; }
__host__ __device__ constexpr int sign_bit(int c, int axis) { return axis == 0 ? sx_of(c) : (axis == 1 ? sy_of(c) : sz_of(c)); }
// Corner with the given sign bits.
__host__ __device__ constexpr int corner_of(int bx, int by, int bz) { return bz * 4 + (by ? (bx ? 2 : 3) : (bx ? 1 : 0)); }
__host__ __device__ constexpr int corner_axes(int axis, int b_axis, int o1, int b1, int o2, int b2)
{
  // corner whose sign bit along `axis` is b_axis, along o1 is b1, along o2 is b2
  return corner_of(axis == 0 ? b_axis : (o1 == 0 ? b1 : b2), axis == 1 ? b_axis : (o1 == 1 ? b1 : b2),
                   axis == 2 ? b_axis : (o1 == 2 ? b1 : b2));
}
// The two axes other than `axis`, in increasing order.
__host__ __device__ constexpr int other1(int axis) { return axis == 0 ? 1 : 0; }
__host__ __device__ constexpr int other2(int axis) { return axis == 2 ? 1 : 2; }

// Reference full-tensor storage slot of row i, column k (K_F_* of
// src/nimble_utils.h:101-109) and symmetric slot (K_S_*, :91-99).
__host__ __device__ constexpr int full_slot(int i, int k)
{
  return i == 0 ? (k == 0 ? 0 : (k == 1 ? 3 : 8)) : (i == 1 ? (k == 0 ? 6 : (k == 1 ? 1 : 4)) : (k == 0 ? 5 : (k == 1 ? 7 : 2)));
}
__host__ __device__ constexpr int sym_slot(int i, int k)
{
  return (i == k) ? i : ((i + k == 1) ? 3 : ((i + k == 3) ? 4 : 5));
}

// Per-step schedule entry: the reference forms t_cur += dt_user, then
// delta = t_cur - t_prev and half = 0.5 * delta
// (src/integrators/explicit_time_integrator.cc:196-199).
struct StepSched {
  double delta;
  double half;
  double time;  // time_current of the step (boundary-condition expressions)
  int    is_output;
  int    pad;
};

// Boundary-condition action on one node, the last one in deck order per
// component (each BC line overwrites the velocity component it names,
// src/nimble_boundary_condition_manager.h:136-217).  kind: 0 none,
// 1 prescribed velocity, 2 prescribed displacement.  expr: -1 for the
// constant value[k], else the index of the expression program f(x, y, z, t)
// that gives it.
struct NodeBC {
  int8_t kind[3];
  int8_t expr[3];
  int8_t pad[2];
  double value[3];
};

// Postfix programs of boundary-condition expressions (bc_expression.cu).
// Constants and variables push; unary operations replace the top; binary
// ones pop one; kExSelect pops two (condition, if-true, if-false).
enum ExprCode : int {
  kExConst, kExX, kExY, kExZ, kExT,
  kExAdd, kExSub, kExMul, kExDiv, kExMod, kExPow,
  kExNeg, kExSin, kExCos, kExTan, kExErf, kExExp, kExLog, kExAbs, kExAsin, kExAcos, kExAtan, kExSqrt, kExCbrt,
  kExErfc, kExCeil, kExRound, kExFloor, kExLog10, kExNot,
  kExGt, kExGe, kExLt, kExLe, kExEq, kExAnd, kExOr, kExXor,
  kExSelect
};
struct ExprOp {
  int    code;
  int    pad;
  double c;  // kExConst
};
constexpr int kExprStack = 16;  // operand stack of the evaluators; deeper programs are refused
__host__ __device__ constexpr bool expr_is_unary(int code) { return code >= kExNeg && code <= kExNot; }

inline int grid_for(long n, int block) { return (int)((n + block - 1) / block); }

// 4-byte asynchronous copies global -> shared (per-thread copy groups), used
// to stage the next element's nodal values while the current one computes.
#ifdef __CUDACC__
__device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
#endif

}  // namespace nsm
