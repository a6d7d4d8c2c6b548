// The reference integrator's explicit loop on host arrays, with the internal
// force from the engine through the host-buffer entry point: the step a
// NimbleSM run makes through the GpuModelData adapter
// (integration/gpu_model_data.h), where ExplicitTimeIntegrator keeps u, v and
// a in host memory and does its O(N) updates on one host thread.
//
// Each step restates src/integrators/explicit_time_integrator.cc:196-276:
//   v += dt/2 a; kinematic conditions; u += dt v; kinematic conditions;
//   f_int = ComputeInternalForce(u) (nsm_compute_internal_force_host);
//   a = (1/m) (f_int + f_ext), f_ext = 0; v += dt/2 a;
//   output step: kinematic conditions.
// The AXPY updates are those of the reference's Viewify operator+=
// (src/nimble_view.h:181-221), and the kinematic conditions those of
// BoundaryConditionManager::ApplyKinematicBC for the explicit scheme
// (src/nimble_boundary_condition_manager.h:148-217) with constant magnitudes.
// Host code only, compiled without FMA contraction: the nodal arithmetic
// rounds as the reference's does, so the state equals the engine's own
// device loop (nsm_advance) bit for bit.
#include <chrono>

#include "../../include/nimble_gb300.h"
#include "nsm_kernels.cuh"

namespace {

void apply_kinematic(const nsm_host_bcs* bc, double t_cur, double t_prev, const double* u, double* v)
{
  if (!bc) return;
  const double delta_t = t_cur - t_prev;
  for (int b = 0; b < bc->num_bcs; b++) {
    const int c = bc->component[b];
    if (bc->kind[b] == NSM_BC_PRESCRIBED_VELOCITY) {
      for (int k = bc->ptr[b]; k < bc->ptr[b + 1]; k++) v[3 * (long)bc->nodes[k] + c] = bc->value[b];
    } else if (bc->kind[b] == NSM_BC_PRESCRIBED_DISPLACEMENT && delta_t > 0.0) {
      for (int k = bc->ptr[b]; k < bc->ptr[b + 1]; k++) {
        const long n = bc->nodes[k];
        v[3 * n + c] = (bc->value[b] - u[3 * n + c]) / delta_t;
      }
    }
  }
}

}  // namespace

extern "C" int nsm_host_loop_steps(nsm_model* model, int num_steps, double* time_current, double dt_user,
                                   int output_frequency, int first_step, int num_load_steps, const double* mass,
                                   const nsm_host_bcs* bcs, double* u, double* v, double* a, double* f_int,
                                   double* host_seconds)
{
  if (!model || !time_current || !mass || !u || !v || !a || !f_int || num_steps < 0)
    return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, "nsm_host_loop_steps: null argument");
  const int N = nsm::model_num_nodes(model);
  if (bcs && bcs->num_bcs > 0) {
    if (!bcs->kind || !bcs->component || !bcs->value || !bcs->ptr || bcs->ptr[0] != 0)
      return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, "nsm_host_loop_steps: incomplete condition table");
    for (int b = 0; b < bcs->num_bcs; b++) {
      if (bcs->kind[b] != NSM_BC_INITIAL_VELOCITY && bcs->kind[b] != NSM_BC_PRESCRIBED_VELOCITY &&
          bcs->kind[b] != NSM_BC_PRESCRIBED_DISPLACEMENT)
        return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, "nsm_host_loop_steps: unknown condition kind");
      if (bcs->component[b] < 0 || bcs->component[b] > 2 || bcs->ptr[b + 1] < bcs->ptr[b])
        return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, "nsm_host_loop_steps: invalid condition");
      if (bcs->ptr[b + 1] > bcs->ptr[b] && !bcs->nodes)
        return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, "nsm_host_loop_steps: null node list");
      for (int k = bcs->ptr[b]; k < bcs->ptr[b + 1]; k++)
        if (bcs->nodes[k] < 0 || bcs->nodes[k] >= N)
          return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, "nsm_host_loop_steps: node id out of range");
    }
  }
  const long n3   = 3L * N;
  double     host = 0.0;
  using clk       = std::chrono::steady_clock;
  for (int s = 0; s < num_steps; s++) {
    const int  step      = first_step + s;
    const bool is_output = output_frequency != 0 && (step % output_frequency == 0 || step == num_load_steps - 1);
    const auto t0        = clk::now();
    const double time_previous = *time_current;
    *time_current += dt_user;
    const double delta_time = *time_current - time_previous;
    const double half       = 0.5 * delta_time;
    for (long i = 0; i < n3; i++) v[i] += half * a[i];
    apply_kinematic(bcs, *time_current, time_previous, u, v);
    for (long i = 0; i < n3; i++) u[i] += delta_time * v[i];
    apply_kinematic(bcs, *time_current, time_previous, u, v);
    const auto t1 = clk::now();
    const int  rc = nsm_compute_internal_force_host(model, u, f_int);
    if (rc != NSM_OK) return rc;
    const auto t2 = clk::now();
    const long N  = n3 / 3;
    for (long i = 0; i < N; i++) {
      const double one_over_m = 1.0 / mass[i];
      a[3 * i]                = one_over_m * (f_int[3 * i] + 0.0);
      a[3 * i + 1]            = one_over_m * (f_int[3 * i + 1] + 0.0);
      a[3 * i + 2]            = one_over_m * (f_int[3 * i + 2] + 0.0);
    }
    for (long i = 0; i < n3; i++) v[i] += half * a[i];
    if (is_output) apply_kinematic(bcs, *time_current, time_previous, u, v);
    const auto t3 = clk::now();
    host += std::chrono::duration<double>(t1 - t0).count() + std::chrono::duration<double>(t3 - t2).count();
  }
  if (host_seconds) *host_seconds = host;
  return NSM_OK;
}
