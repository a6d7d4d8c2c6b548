// Node kernels: assembly of the element forces and the central-difference
// update.
//
// FP64 form: every product and sum is an explicit round-to-nearest intrinsic
// (__dmul_rn / __dadd_rn are never fused), so given the same element forces
// the nodal state equals the reference's bit for bit.  FP32-mixed form: the
// FP32 element forces are assembled in FP32 and the FP64 update uses fused
// multiply-adds -- on this chip FP64 operations, not bytes, bound a node
// update, and the exact rounding of the reference buys nothing when the forces
// themselves are FP32.
#include "nsm_kernels.cuh"

namespace nsm {

// Value of expression program `prog` at node n and time t: the postfix
// program on an operand stack, one double-precision operation at a time (no
// contraction across operations).  The host refuses programs deeper than the
// stack; a malformed one gives NaN rather than an access outside it.
__device__ __noinline__ double eval_bc_expression(const BcExprTable& ex, int prog, int n, double t)
{
  const double x = ex.X[n], y = ex.X[ex.ld_n + n], z = ex.X[2 * ex.ld_n + n];
  double       st[kExprStack];
  int          sp = 0;
  for (int i = ex.start[prog]; i < ex.start[prog + 1]; i++) {
    const ExprOp o = ex.code[i];
    if (o.code <= kExT) {
      if (sp >= kExprStack) return NAN;
      st[sp++] = o.code == kExConst ? o.c : (o.code == kExX ? x : (o.code == kExY ? y : (o.code == kExZ ? z : t)));
      continue;
    }
    if (o.code == kExSelect) {
      if (sp < 3) return NAN;
      sp -= 2;
      st[sp - 1] = st[sp - 1] != 0.0 ? st[sp] : st[sp + 1];
      continue;
    }
    if (expr_is_unary(o.code)) {
      if (sp < 1) return NAN;
      const double a = st[sp - 1];
      double       r;
      switch (o.code) {
        case kExNeg: r = -a; break;
        case kExSin: r = sin(a); break;
        case kExCos: r = cos(a); break;
        case kExTan: r = tan(a); break;
        case kExErf: r = erf(a); break;
        case kExExp: r = exp(a); break;
        case kExLog: r = log(a); break;
        case kExAbs: r = fabs(a); break;
        case kExAsin: r = asin(a); break;
        case kExAcos: r = acos(a); break;
        case kExAtan: r = atan(a); break;
        case kExSqrt: r = sqrt(a); break;
        case kExCbrt: r = cbrt(a); break;
        case kExErfc: r = erfc(a); break;
        case kExCeil: r = ceil(a); break;
        case kExRound: r = round(a); break;
        case kExFloor: r = floor(a); break;
        case kExLog10: r = log10(a); break;
        default: r = a != 0.0 ? 0.0 : 1.0; break;  // kExNot
      }
      st[sp - 1] = r;
      continue;
    }
    if (sp < 2) return NAN;
    const double a = st[sp - 2], b = st[sp - 1];
    double       r;
    switch (o.code) {
      case kExAdd: r = __dadd_rn(a, b); break;
      case kExSub: r = __dsub_rn(a, b); break;
      case kExMul: r = __dmul_rn(a, b); break;
      case kExDiv: r = __ddiv_rn(a, b); break;
      case kExMod: r = fmod(a, b); break;
      case kExPow: r = pow(a, b); break;
      case kExGt: r = a > b ? 1.0 : 0.0; break;
      case kExGe: r = a >= b ? 1.0 : 0.0; break;
      case kExLt: r = a < b ? 1.0 : 0.0; break;
      case kExLe: r = a <= b ? 1.0 : 0.0; break;
      case kExEq: r = a == b ? 1.0 : 0.0; break;
      case kExAnd: r = (a != 0.0 && b != 0.0) ? 1.0 : 0.0; break;
      case kExOr: r = (a != 0.0 || b != 0.0) ? 1.0 : 0.0; break;
      case kExXor: r = ((a != 0.0) != (b != 0.0)) ? 1.0 : 0.0; break;
      default: return NAN;
    }
    st[--sp - 1] = r;
  }
  return sp == 1 ? st[0] : NAN;
}

// ApplyKinematicBC for the explicit scheme
// (src/nimble_boundary_condition_manager.h:136-217): prescribed velocity sets
// v; prescribed displacement sets v = (d - u) / delta when delta > 0.  The
// magnitude is the line's constant or its expression's value at the node's
// reference coordinates and time_current (`ev`, evaluated beforehand).
__device__ __forceinline__ void apply_bc(const NodeBC& bc, double delta, const double* ev, const double u[3],
                                         double v[3])
{
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (bc.kind[k] == 0 || (bc.kind[k] == 2 && !(delta > 0.0))) continue;
    const double value = bc.expr[k] < 0 ? bc.value[k] : ev[k];
    if (bc.kind[k] == 1) {
      v[k] = value;
    } else {
      v[k] = __ddiv_rn(__dadd_rn(value, -u[k]), delta);
    }
  }
}

// f + 0.0, the zero external force added as the reference adds it, without
// the FP64 pipe: the sum is f itself except for -0.0, which becomes +0.0.
__device__ __forceinline__ double plus_zero(double f)
{
  return __double_as_longlong(f) == (long long)0x8000000000000000ULL ? 0.0 : f;
}

// y + s*x, rounded as the reference's two operations or fused.
template <bool kExact>
__device__ __forceinline__ double axpy(double s, double x, double y)
{
  return kExact ? __dadd_rn(y, __dmul_rn(s, x)) : fma(s, x, y);
}

// The assembled element force of node n: element contributions in increasing
// element order, from the corner-major planes fe[(3 c + i) ld_e + e] (a row
// of consecutive nodes reads consecutive elements of one plane per slot).
template <typename TF, bool kExact>
__device__ __forceinline__ void gather_force(const NodeArgs& a, int n, double f[3])
{
  const TF* fe    = reinterpret_cast<const TF*>(a.fe);
  TF        fs[3] = {TF(0), TF(0), TF(0)};
  // the first 8 incidences (all of them at a hex mesh's interior node) from
  // the slot-major copy: every load issued before the first sum, the sums in
  // the same order as the rest from the CSR below
  constexpr int  kFirst = 8;
  const bool     more   = (__ldg(&a.node_more[n >> 5]) >> (n & 31)) & 1u;
  int            ec[kFirst];
#pragma unroll
  for (int j = 0; j < kFirst; j++) ec[j] = __ldg(&a.node_slots[(long)j * a.ld_n + n]);
  TF x[kFirst][3];
#pragma unroll
  for (int j = 0; j < kFirst; j++)
#pragma unroll
    for (int i = 0; i < 3; i++)
      x[j][i] = ec[j] >= 0 ? __ldg(&fe[((ec[j] & 7) * 3 + i) * a.ld_e + (ec[j] >> 3)]) : TF(0);
  // the first sum is 0 + x: x itself but for -0.0 (+0.0), an integer select
  // rather than an FP64 add in the exact form
  if (ec[0] >= 0) {
#pragma unroll
    for (int i = 0; i < 3; i++) fs[i] = kExact ? TF(plus_zero(double(x[0][i]))) : fs[i] + x[0][i];
  }
#pragma unroll
  for (int j = 1; j < kFirst; j++)
    if (ec[j] >= 0) {
#pragma unroll
      for (int i = 0; i < 3; i++) fs[i] = kExact ? TF(__dadd_rn(double(fs[i]), double(x[j][i]))) : fs[i] + x[j][i];
    }
  const int k1 = more ? __ldg(&a.node_ptr[n + 1]) : 0;
  for (int k = more ? __ldg(&a.node_ptr[n]) + kFirst : 0; k < k1; k++) {
    const int  ec = __ldg(&a.node_inc[k]);
    const long e  = ec >> 3;
    const int  c  = ec & 7;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const TF xi = __ldg(&fe[(c * 3 + i) * a.ld_e + e]);
      fs[i]       = kExact ? TF(__dadd_rn(double(fs[i]), double(xi))) : fs[i] + xi;
    }
  }
#pragma unroll
  for (int i = 0; i < 3; i++) f[i] = double(fs[i]);
}

template <typename TF, bool kExact>
__global__ void __launch_bounds__(256, sizeof(TF) == 4 ? 5 : 4) k_node_update(NodeArgs a)
{
  const int n = a.n_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const long ld = a.ld_n;
  double     u[3], v[3], acc[3];
  const int  slot  = a.bc_slot[n];
  const int  group = a.node_group ? __ldg(&a.node_group[n]) : 0;
  NodeBC     bc;
  if (slot >= 0) bc = a.bcs[slot];

  if (a.k_post >= 0 || a.gather_only) {
    // ModelData::ComputeInternalForce: zero, then element contributions in
    // increasing element order (src/nimble_model_data.cc:620-667,
    // src/nimble_block.cc:373-383).
    double f[3];
    if (a.closure && group >= a.closure_first) {
      // UqModel::ApplyClosure (src/uq/nimble_uq.cc:327-345): f = f_0 c_0, then
      // f += f_k c_k over the exact samples, from the same assembled forces
      // the nominal and exact samples' own nodes compute
      const int     local = n - a.node_off[group];
      const double* c     = a.closure + (long)(group - a.closure_first) * (a.num_exact + 1);
      double        fk[3];
      gather_force<TF, kExact>(a, a.node_off[0] + local, fk);
#pragma unroll
      for (int i = 0; i < 3; i++) f[i] = kExact ? __dmul_rn(fk[i], c[0]) : fk[i] * c[0];
      for (int k = 1; k <= a.num_exact; k++) {
        gather_force<TF, kExact>(a, a.node_off[k] + local, fk);
#pragma unroll
        for (int i = 0; i < 3; i++) f[i] = kExact ? __dadd_rn(f[i], __dmul_rn(fk[i], c[k])) : fma(fk[i], c[k], f[i]);
      }
    } else {
      gather_force<TF, kExact>(a, n, f);
    }
    // f_int (and a, below) are read by nothing inside a launch sequence: the
    // sequence's last launch (k_pre < 0) leaves them for the host's queries
    if (a.gather_only || a.k_pre < 0) {
#pragma unroll
      for (int i = 0; i < 3; i++) a.f_int[i * ld + n] = f[i];
    }
    if (a.gather_only) return;
    const StepSched s  = a.sched[(long)(*a.step_base + a.k_post) * a.num_groups + group];
    const double    im = a.inv_mass[n];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      // a = (1/m) (f_int + f_ext), f_ext = 0 (src/integrators/explicit_time_integrator.cc:250-257)
      acc[i] = kExact ? __dmul_rn(im, plus_zero(f[i])) : im * f[i];
      v[i]   = axpy<kExact>(s.half, acc[i], a.v[i * ld + n]);
      u[i]   = a.u[i * ld + n];
    }
    if (s.is_output && slot >= 0) apply_bc(bc, s.delta, a.bc_expr_val ? a.bc_expr_val + (long)slot * 3 : nullptr, u, v);
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      acc[i] = a.a[i * ld + n];
      v[i]   = a.v[i * ld + n];
      u[i]   = a.u[i * ld + n];
    }
  }
  if (a.k_pre >= 0) {
    // v^{n+1/2} = v^n + dt/2 a^n; BCs; u^{n+1} = u^n + dt v^{n+1/2}; BCs
    // (src/integrators/explicit_time_integrator.cc:200-223)
    const StepSched s = a.sched[(long)(*a.step_base + a.k_pre) * a.num_groups + group];
#pragma unroll
    for (int i = 0; i < 3; i++) v[i] = axpy<kExact>(s.half, acc[i], v[i]);
    const double* ev = a.bc_expr_val ? a.bc_expr_val + ((long)a.num_bc_slots + slot) * 3 : nullptr;
    if (slot >= 0) apply_bc(bc, s.delta, ev, u, v);
#pragma unroll
    for (int i = 0; i < 3; i++) u[i] = axpy<kExact>(s.delta, v[i], u[i]);
    if (slot >= 0) apply_bc(bc, s.delta, ev, u, v);
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    a.u[i * ld + n] = u[i];
    a.v[i * ld + n] = v[i];
    if (a.k_post >= 0 && a.k_pre < 0) a.a[i * ld + n] = acc[i];
    if (sizeof(TF) == 4 && a.uf != nullptr) a.uf[i * ld + n] = (float)u[i];  // FP32 forms only
  }
}

cudaError_t launch_node_update(const NodeArgs& a, cudaStream_t stream)
{
  if (a.N <= a.n_begin) return cudaSuccess;
  if (a.fe_is_float)
    k_node_update<float, false><<<grid_for(a.N - a.n_begin, 256), 256, 0, stream>>>(a);
  else
    k_node_update<double, true><<<grid_for(a.N - a.n_begin, 256), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

__global__ void k_bc_expr_values(NodeArgs a, const int* __restrict__ slot_node, BcExprTable ex, double* __restrict__ out)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.num_bc_slots) return;
  const NodeBC bc    = a.bcs[s];
  const int    n     = slot_node[s];
  const int    group = a.node_group ? a.node_group[n] : 0;
  for (int level = 0; level < 2; level++) {
    const int k = level == 0 ? a.k_post : a.k_pre;
    if (k < 0) continue;
    const double t = a.sched[(long)(*a.step_base + k) * a.num_groups + group].time;
    for (int c = 0; c < 3; c++)
      if (bc.expr[c] >= 0) out[((long)level * a.num_bc_slots + s) * 3 + c] = eval_bc_expression(ex, bc.expr[c], n, t);
  }
}

cudaError_t launch_bc_expr_values(const NodeArgs& a, const int* slot_node, const BcExprTable& ex, double* out,
                                  cudaStream_t stream)
{
  if (a.num_bc_slots == 0) return cudaSuccess;
  k_bc_expr_values<<<grid_for(a.num_bc_slots, 128), 128, 0, stream>>>(a, slot_node, ex, out);
  return cudaGetLastError();
}

__global__ void k_advance_base(int* base, int k) { *base += k; }

cudaError_t launch_advance_base(int* step_base, int k, cudaStream_t stream)
{
  k_advance_base<<<1, 1, 0, stream>>>(step_base, k);
  return cudaGetLastError();
}

__global__ void k_apply_bc(int N, long ld_n, const int* __restrict__ bc_slot, const NodeBC* __restrict__ bcs,
                           double delta, double time, BcExprTable ex, const double* __restrict__ u,
                           double* __restrict__ v)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int slot = bc_slot[n];
  if (slot < 0) return;
  double uu[3], vv[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    uu[i] = u[i * ld_n + n];
    vv[i] = v[i * ld_n + n];
  }
  const NodeBC& bc = bcs[slot];
  double        ev[3];
#pragma unroll
  for (int k = 0; k < 3; k++) ev[k] = bc.expr[k] >= 0 ? eval_bc_expression(ex, bc.expr[k], n, time) : 0.0;
  apply_bc(bc, delta, ev, uu, vv);
#pragma unroll
  for (int i = 0; i < 3; i++) v[i * ld_n + n] = vv[i];
}

cudaError_t launch_apply_bc(int N, long ld_n, const int* bc_slot, const NodeBC* bcs, double delta, double time,
                            const BcExprTable& ex, const double* u, double* v, cudaStream_t stream)
{
  if (N == 0) return cudaSuccess;
  k_apply_bc<<<grid_for(N, 256), 256, 0, stream>>>(N, ld_n, bc_slot, bcs, delta, time, ex, u, v);
  return cudaGetLastError();
}

}  // namespace nsm
