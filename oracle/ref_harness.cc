/* Reference harness: drives NimbleSM's own host objects (compiled from the
 * reference sources by oracle/Makefile) on an in-memory mesh.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product: it
 * is linked only into oracle/_ref/libnimble_ref.so and is loaded only by the
 * tests and by tests/golden/make_golden.py.  (bench.py's CPU baseline is the
 * C restatement, oracle/nsm_oracle.c, which is bitwise this code's result and
 * builds on any host.)
 *
 * What it runs is the reference's code: nimble::DataManager,
 * nimble::ModelData, nimble::Block, nimble::HexElement and
 * nimble::NeohookeanMaterial.  The only restated part is the explicit time
 * loop, because its class (ExplicitTimeIntegrator) needs NimbleApplication,
 * which cannot be built without Kokkos and Exodus.  The restatement follows
 * src/integrators/explicit_time_integrator.cc:123-278 statement by statement,
 * without contact and without Exodus output.
 */
#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "nimble_boundary_condition_manager.h"
#include "nimble_data_manager.h"
#include "nimble_element.h"
#include "nimble_expression_parser.h"
#include "nimble_genesis_mesh.h"
#include "nimble_material.h"
#include "nimble_material_factory.h"
#include "nimble_model_data.h"
#include "nimble_parser.h"
#include "nimble_view.h"

namespace {

// Fills the protected members of the reference's mesh class
// (src/nimble_genesis_mesh.h:328-354) directly, as ReadTextFile does
// (src/nimble_genesis_mesh.cc:318-427), but from memory: blocks with ids
// 1..num_blocks (elem_block [E] 0-based block of each element, or null for
// one block).
class HarnessMesh : public nimble::GenesisMesh
{
 public:
  void
  Fill(
      int                             num_nodes,
      const double*                   xyz,
      int                             num_elem,
      const int*                      conn,
      int                             num_node_sets,
      const int*                      ns_ptr,
      const int*                      ns_nodes,
      const std::vector<std::string>& ns_names,
      int                             num_blocks = 1,
      const int*                      elem_block = nullptr)
  {
    file_name_ = "in_memory";
    dim_       = 3;
    node_global_id_.resize(num_nodes);
    node_x_.resize(num_nodes);
    node_y_.resize(num_nodes);
    node_z_.resize(num_nodes);
    for (int i = 0; i < num_nodes; i++) {
      node_global_id_[i] = i;
      node_x_[i]         = xyz[3 * i];
      node_y_[i]         = xyz[3 * i + 1];
      node_z_[i]         = xyz[3 * i + 2];
    }
    elem_global_id_.resize(num_elem);
    for (int e = 0; e < num_elem; e++) elem_global_id_[e] = e;
    for (int b = 0; b < num_blocks; b++) {
      const int id = b + 1;
      block_ids_.push_back(id);
      all_block_ids_.push_back(id);
      block_names_[id]              = "block_" + std::to_string(id);
      all_block_names_[id]          = block_names_[id];
      block_num_nodes_per_elem_[id] = 8;
      block_elem_global_ids_[id]    = std::vector<int>();
      block_elem_connectivity_[id]  = std::vector<int>();
    }
    for (int e = 0; e < num_elem; e++) {
      const int id = (elem_block ? elem_block[e] : 0) + 1;
      block_elem_global_ids_[id].push_back(e);
      block_elem_connectivity_[id].insert(block_elem_connectivity_[id].end(), conn + 8 * static_cast<size_t>(e),
                                          conn + 8 * static_cast<size_t>(e) + 8);
    }
    for (int s = 0; s < num_node_sets; s++) {
      int id = s + 1;
      node_set_ids_.push_back(id);
      node_set_names_[id] = ns_names[s];
      node_sets_[id]      = std::vector<int>(ns_nodes + ns_ptr[s], ns_nodes + ns_ptr[s + 1]);
    }
  }
};

// Feeds input-deck lines to the reference parser (src/nimble_parser.cc:239-326).
class HarnessParser : public nimble::Parser
{
 public:
  void
  Set(const std::string& key, const std::string& value)
  {
    ParseKeyValue(key, value);
  }
};

// Exposes the reference's per-point neo-Hookean stress
// (NeohookeanMaterial::GetStress, src/nimble_material.cc:252-310), which the
// batched form (src/nimble_material.cc:226-250) calls once per point.
class PointNeohookean : public nimble::NeohookeanMaterial
{
 public:
  using nimble::NeohookeanMaterial::NeohookeanMaterial;
  void
  Stress(int num_pts, const double* F, double* sigma) const
  {
    nimble::Viewify<1, const double> null_view;
    for (int pt = 0; pt < num_pts; pt++) {
      nimble::Viewify<1, const double> def_grad(&F[9 * pt], 9);
      GetStress(0.0, 0.0, null_view, def_grad, null_view, {&sigma[6 * pt], 6});
    }
  }
};

PointNeohookean
MakeNeohookean(double density, double bulk_modulus, double shear_modulus)
{
  nimble::MaterialParameters params;
  params.AddParameter("density", density);
  params.AddParameter("bulk_modulus", bulk_modulus);
  params.AddParameter("shear_modulus", shear_modulus);
  return PointNeohookean(params);
}

std::vector<std::string>
SplitLines(const char* s)
{
  std::vector<std::string> out;
  if (s == nullptr) return out;
  std::stringstream ss(s);
  std::string       line;
  while (std::getline(ss, line)) {
    if (!line.empty()) out.push_back(line);
  }
  return out;
}

thread_local std::string g_last_error;

}  // namespace

extern "C" {

const char*
nimref_last_error()
{
  return g_last_error.c_str();
}

/* Runs `num_steps` explicit steps of the reference on the given mesh.
 *
 * xyz[3N], conn[8E] (0-based, reference corner order); elem_block [E]
 * (0-based block of each element, non-decreasing; null: one block) with one
 * '\n'-separated material line per block as in an input deck ("<model>
 * density .. bulk_modulus .. shear_modulus .."); node sets in CSR form
 * (ns_ptr[num_node_sets+1], ns_nodes) with '\n'-separated names;
 * '\n'-separated boundary-condition lines.  v_init (nullable, [N][3]) is
 * written into the velocity after ApplyInitialConditions and before
 * ApplyKinematicConditions(0,0).
 *
 * The state is recorded after every output step of the schedule (the steps
 * the reference writes, src/integrators/explicit_time_integrator.cc:192-194;
 * only the last step when output_frequency is 0), at most max_outputs of
 * them, into out_* arrays laid out [output][...]: u, v, a, f_int [N][3]; F
 * [E][8][9] and sigma [E][8][6] in the reference component order, copied
 * from the element data the reference stored in that step (nullable).
 * Also the lumped mass [N], the critical time step, the wall seconds of the
 * step loop and the number of recorded outputs.  Returns 0, or -1 with
 * nimref_last_error() set. */
static int
run_impl(
    int           num_nodes,
    const double* xyz,
    int           num_elem,
    const int*    conn,
    int           num_blocks,
    const int*    elem_block,
    const char*   materials,
    int           num_node_sets,
    const int*    ns_ptr,
    const int*    ns_nodes,
    const char*   ns_names,
    const char*   bcs,
    double        final_time,
    int           num_steps,
    int           output_frequency,
    const double* v_init,
    int           max_outputs,
    double*       out_u,
    double*       out_v,
    double*       out_a,
    double*       out_fint,
    double*       out_F,
    double*       out_sigma,
    double*       out_mass,
    double*       out_dt_crit,
    double*       out_loop_seconds,
    int*          out_num_outputs,
    const char*   uq_params,     // "uq parameters" lines, or null (no UQ)
    const char*   uq_samples,    // the UQ samples file
    int           num_samples,   // exact + approximate samples expected
    double*       out_su,        // [output][sample][N][3], exact samples first
    double*       out_sv,
    double*       out_sf)
{
  try {
    HarnessMesh mesh;
    mesh.Fill(num_nodes, xyz, num_elem, conn, num_node_sets, ns_ptr, ns_nodes, SplitLines(ns_names), num_blocks,
              elem_block);

    HarnessParser parser;
    {
      // std::to_string truncates to 6 digits; the deck value is parsed by atof.
      std::ostringstream os;
      os.precision(17);
      os << final_time;
      parser.Set("final time", os.str());
    }
    parser.Set("number of load steps", std::to_string(num_steps));
    parser.Set("output frequency", std::to_string(output_frequency));
    auto mat_lines = SplitLines(materials);
    if (static_cast<int>(mat_lines.size()) != num_blocks) throw std::invalid_argument("one material line per block");
    for (int b = 0; b < num_blocks; b++) {
      const std::string id = std::to_string(b + 1);
      parser.Set("material parameters", "material_" + id + " " + mat_lines[b]);
      parser.Set("element block", "block_" + id + " material_" + id);
    }
    parser.Set("output fields", "displacement");
    for (auto const& bc : SplitLines(bcs)) parser.Set("boundary condition", bc);
    if (uq_params) {
#ifdef NIMBLE_HAVE_UQ
      parser.SetToUseUQ();  // what the command line's UQ flag sets (src/nimble_parser.h:276-279)
      for (auto const& line : SplitLines(uq_params)) parser.Set("uq parameters", line);
      parser.Set("uq model", std::string("file ") + uq_samples);
#else
      throw std::invalid_argument("library compiled without the UQ mode");
#endif
    }

    nimble::DataManager data_manager(parser, mesh);
    auto                model_data_ptr = data_manager.GetModelData();
    auto&               model_data     = *model_data_ptr;
    model_data.InitializeBlocks(data_manager, std::make_shared<nimble::MaterialFactory>());
    auto& host_model = *std::dynamic_pointer_cast<nimble::ModelData>(model_data_ptr);

    // ---- src/integrators/explicit_time_integrator.cc:104-147 ----
    auto displacement   = model_data.GetVectorNodeData("displacement");
    auto velocity       = model_data.GetVectorNodeData("velocity");
    auto acceleration   = model_data.GetVectorNodeData("acceleration");
    auto internal_force = model_data.GetVectorNodeData("internal_force");
    auto external_force = model_data.GetVectorNodeData("external_force");

    model_data.ComputeLumpedMass(data_manager);
    double     critical_time_step = model_data.GetCriticalTimeStep();
    auto const lumped_mass        = model_data.GetScalarNodeData("lumped_mass");

    double initial_time             = parser.InitialTime();
    double time_current             = initial_time;
    double time_previous            = initial_time;
    double delta_time               = 0.0;
    double half_delta_time          = 0.0;
    int    num_load_steps           = parser.NumLoadSteps();
    double user_specified_time_step = (parser.FinalTime() - initial_time) / num_load_steps;

    // UQ trajectories (nimble_uq::ModelData, src/uq/nimble_uq.cc:282-326):
    // exact samples, then approximate samples
    std::vector<double*> su, sv, sf;
    if (uq_params) {
      const char* kinds[2] = {"exact", "sample"};
      for (const char* kind : kinds) {
        for (int i = 1;; i++) {
          const std::string tag = "_" + std::to_string(i);
          const int         id  = host_model.GetFieldId(std::string(kind) + "_displacement" + tag);
          if (id < 0) break;
          su.push_back(host_model.GetNodeData(id));
          sv.push_back(host_model.GetNodeData(host_model.GetFieldId(std::string(kind) + "_velocity" + tag)));
          sf.push_back(host_model.GetNodeData(host_model.GetFieldId(std::string(kind) + "_force" + tag)));
        }
      }
      if (static_cast<int>(su.size()) != num_samples) throw std::invalid_argument("unexpected number of UQ samples");
    }

    model_data.ApplyInitialConditions(data_manager);
    if (v_init != nullptr) {
      // the initial velocity of every trajectory, as an initial_velocity
      // condition would set it (src/nimble_boundary_condition_manager.h:93-123)
      for (int i = 0; i < num_nodes; i++)
        for (int k = 0; k < 3; k++) {
          velocity(i, k) = v_init[3 * i + k];
          for (double* s_v : sv) s_v[3 * i + k] = v_init[3 * i + k];
        }
    }
    model_data.ApplyKinematicConditions(data_manager, 0.0, 0.0);

    // The state after a step: nodal fields, and F and sigma of every point
    // from the element data stored in the step (after UpdateStates the
    // newest values are the "n" data; per element 8 points x [F(9), sigma(6)],
    // src/nimble_block.cc:85-108).
    int  recorded = 0;
    auto record   = [&]() {
      if (recorded >= max_outputs) return;
      const size_t o = static_cast<size_t>(recorded);
      for (int i = 0; i < num_nodes; i++) {
        for (int k = 0; k < 3; k++) {
          const size_t j = o * 3 * num_nodes + 3 * i + k;
          if (out_u) out_u[j] = displacement(i, k);
          if (out_v) out_v[j] = velocity(i, k);
          if (out_a) out_a[j] = acceleration(i, k);
          if (out_fint) out_fint[j] = internal_force(i, k);
        }
      }
      for (size_t smp = 0; smp < su.size(); smp++) {
        const size_t base = (o * su.size() + smp) * 3 * static_cast<size_t>(num_nodes);
        if (out_su) std::memcpy(out_su + base, su[smp], 3 * sizeof(double) * num_nodes);
        if (out_sv) std::memcpy(out_sv + base, sv[smp], 3 * sizeof(double) * num_nodes);
        if (out_sf) std::memcpy(out_sf + base, sf[smp], 3 * sizeof(double) * num_nodes);
      }
      if (out_F || out_sigma) {
        for (int b = 0; b < num_blocks; b++) {
          const std::vector<double>& data = host_model.GetElementDataOld(b + 1);
          const std::vector<int>&    ids  = mesh.GetElementGlobalIdsInBlock(b + 1);
          const size_t               per  = data.size() / (ids.empty() ? 1 : ids.size()) / 8;
          for (size_t le = 0; le < ids.size(); le++) {
            const size_t e = static_cast<size_t>(ids[le]);
            for (int ip = 0; ip < 8; ip++) {
              const double* src = &data[(le * 8 + ip) * per];
              if (out_F) std::memcpy(out_F + o * 72 * num_elem + 72 * e + 9 * ip, src, 9 * sizeof(double));
              if (out_sigma) std::memcpy(out_sigma + o * 48 * num_elem + 48 * e + 6 * ip, src + 9, 6 * sizeof(double));
            }
          }
        }
      }
      recorded++;
    };

    auto t0 = std::chrono::steady_clock::now();
    // ---- src/integrators/explicit_time_integrator.cc:177-278 ----
    for (int step = 0; step < num_load_steps; step++) {
      bool is_output_step = false;
      if (output_frequency != 0) {
        if (step % output_frequency == 0 || step == num_load_steps - 1) { is_output_step = true; }
      }
      time_previous = time_current;
      time_current += user_specified_time_step;
      delta_time      = time_current - time_previous;
      half_delta_time = 0.5 * delta_time;

      velocity += half_delta_time * acceleration;
      model_data.UpdateWithNewVelocity(data_manager, half_delta_time);
      model_data.ApplyKinematicConditions(data_manager, time_current, time_previous);

      displacement += delta_time * velocity;
      model_data.UpdateWithNewDisplacement(data_manager, delta_time);
      model_data.ApplyKinematicConditions(data_manager, time_current, time_previous);

      model_data.ComputeExternalForce(data_manager, time_previous, time_current, is_output_step);
      model_data.ComputeInternalForce(
          data_manager, time_previous, time_current, is_output_step, displacement, internal_force);

      for (int i = 0; i < num_nodes; ++i) {
        const double oneOverM = 1.0 / lumped_mass(i);
        acceleration(i, 0)    = oneOverM * (internal_force(i, 0) + external_force(i, 0));
        acceleration(i, 1)    = oneOverM * (internal_force(i, 1) + external_force(i, 1));
        acceleration(i, 2)    = oneOverM * (internal_force(i, 2) + external_force(i, 2));
      }
      velocity += half_delta_time * acceleration;
      model_data.UpdateWithNewVelocity(data_manager, half_delta_time);

      if (is_output_step) { model_data.ApplyKinematicConditions(data_manager, time_current, time_previous); }
      model_data.UpdateStates(data_manager);
      if (is_output_step || (output_frequency == 0 && step == num_load_steps - 1)) record();
    }
    auto t1 = std::chrono::steady_clock::now();

    if (out_loop_seconds) *out_loop_seconds = std::chrono::duration<double>(t1 - t0).count();
    if (out_dt_crit) *out_dt_crit = critical_time_step;
    if (out_mass)
      for (int i = 0; i < num_nodes; i++) out_mass[i] = lumped_mass(i);
    if (out_num_outputs) *out_num_outputs = recorded;
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  }
}

int
nimref_run_blocks(
    int           num_nodes,
    const double* xyz,
    int           num_elem,
    const int*    conn,
    int           num_blocks,
    const int*    elem_block,
    const char*   materials,
    int           num_node_sets,
    const int*    ns_ptr,
    const int*    ns_nodes,
    const char*   ns_names,
    const char*   bcs,
    double        final_time,
    int           num_steps,
    int           output_frequency,
    const double* v_init,
    int           max_outputs,
    double*       out_u,
    double*       out_v,
    double*       out_a,
    double*       out_fint,
    double*       out_F,
    double*       out_sigma,
    double*       out_mass,
    double*       out_dt_crit,
    double*       out_loop_seconds,
    int*          out_num_outputs)
{
  return run_impl(num_nodes, xyz, num_elem, conn, num_blocks, elem_block, materials, num_node_sets, ns_ptr, ns_nodes,
                  ns_names, bcs, final_time, num_steps, output_frequency, v_init, max_outputs, out_u, out_v, out_a,
                  out_fint, out_F, out_sigma, out_mass, out_dt_crit, out_loop_seconds, out_num_outputs, nullptr,
                  nullptr, 0, nullptr, nullptr, nullptr);
}

#ifdef NIMBLE_HAVE_UQ
/* The reference's UQ mode (nimble_uq::ModelData, src/uq/nimble_uq_model_data.cc:145-248,
 * and UqModel, src/uq/nimble_uq.cc): as nimref_run_blocks, with the
 * "uq parameters" lines (one per material, "material_<b> <param> <range> ...")
 * and the samples file (src/uq/nimble_uq.cc:145-218).  The nominal
 * trajectory is out_u / out_v / out_fint; out_su, out_sv, out_sf
 * [output][sample][N][3] hold the exact samples and then the approximate
 * samples (num_samples in all).  v_init, when given, is every trajectory's
 * initial velocity.  The reference writes parameter_samples.dat into the
 * working directory. */
int
nimref_run_uq(
    int           num_nodes,
    const double* xyz,
    int           num_elem,
    const int*    conn,
    int           num_blocks,
    const int*    elem_block,
    const char*   materials,
    int           num_node_sets,
    const int*    ns_ptr,
    const int*    ns_nodes,
    const char*   ns_names,
    const char*   bcs,
    double        final_time,
    int           num_steps,
    int           output_frequency,
    const double* v_init,
    const char*   uq_params,
    const char*   uq_samples,
    int           num_samples,
    int           max_outputs,
    double*       out_u,
    double*       out_v,
    double*       out_fint,
    double*       out_su,
    double*       out_sv,
    double*       out_sf,
    double*       out_mass,
    double*       out_dt_crit,
    int*          out_num_outputs)
{
  return run_impl(num_nodes, xyz, num_elem, conn, num_blocks, elem_block, materials, num_node_sets, ns_ptr, ns_nodes,
                  ns_names, bcs, final_time, num_steps, output_frequency, v_init, max_outputs, out_u, out_v, nullptr,
                  out_fint, nullptr, nullptr, out_mass, out_dt_crit, nullptr, out_num_outputs, uq_params, uq_samples,
                  num_samples, out_su, out_sv, out_sf);
}
#endif

/* One block of one material; the state after the last step only (see
 * nimref_run_blocks).  material: "<model> density .. bulk_modulus .. shear_modulus ..". */
int
nimref_run(
    int           num_nodes,
    const double* xyz,
    int           num_elem,
    const int*    conn,
    int           num_node_sets,
    const int*    ns_ptr,
    const int*    ns_nodes,
    const char*   ns_names,
    const char*   material,
    const char*   bcs,
    double        final_time,
    int           num_steps,
    int           output_frequency,
    const double* v_init,
    double*       out_u,
    double*       out_v,
    double*       out_a,
    double*       out_fint,
    double*       out_F,
    double*       out_sigma,
    double*       out_mass,
    double*       out_dt_crit,
    double*       out_loop_seconds)
{
  std::vector<double> u, v, a, f, F, S;
  int                 n = 0;
  const int           max_out =
      output_frequency == 0 ? 1 : (num_steps + output_frequency - 1) / output_frequency + 1;
  if (out_u) u.resize(static_cast<size_t>(max_out) * 3 * num_nodes);
  if (out_v) v.resize(static_cast<size_t>(max_out) * 3 * num_nodes);
  if (out_a) a.resize(static_cast<size_t>(max_out) * 3 * num_nodes);
  if (out_fint) f.resize(static_cast<size_t>(max_out) * 3 * num_nodes);
  if (out_F) F.resize(static_cast<size_t>(max_out) * 72 * num_elem);
  if (out_sigma) S.resize(static_cast<size_t>(max_out) * 48 * num_elem);
  auto p  = [](std::vector<double>& x) { return x.empty() ? nullptr : x.data(); };
  int  rc = nimref_run_blocks(num_nodes, xyz, num_elem, conn, 1, nullptr, material, num_node_sets, ns_ptr, ns_nodes,
                             ns_names, bcs, final_time, num_steps, output_frequency, v_init, max_out, p(u), p(v),
                             p(a), p(f), p(F), p(S), out_mass, out_dt_crit, out_loop_seconds, &n);
  if (rc != 0 || n == 0) return rc != 0 ? rc : -1;
  const size_t last = static_cast<size_t>(n - 1);
  auto         copy = [&](double* dst, std::vector<double>& src, size_t per) {
    if (dst) std::memcpy(dst, src.data() + last * per, per * sizeof(double));
  };
  copy(out_u, u, 3 * static_cast<size_t>(num_nodes));
  copy(out_v, v, 3 * static_cast<size_t>(num_nodes));
  copy(out_a, a, 3 * static_cast<size_t>(num_nodes));
  copy(out_fint, f, 3 * static_cast<size_t>(num_nodes));
  copy(out_F, F, 72 * static_cast<size_t>(num_elem));
  copy(out_sigma, S, 48 * static_cast<size_t>(num_elem));
  return 0;
}

/* One element through the reference: deformation gradients, neo-Hookean
 * stress and nodal forces, exactly as the block functor calls them
 * (src/nimble_block.cc:309-372).  X and u are [8][3]; F [8][9], sigma [8][6],
 * f [8][3] (the element's contribution that is added into f_int). */
int
nimref_element(
    const double* X,
    const double* u,
    double        density,
    double        bulk_modulus,
    double        shear_modulus,
    double*       F,
    double*       sigma,
    double*       f)
{
  try {
    nimble::HexElement element;
    auto               nh = MakeNeohookean(density, bulk_modulus, shear_modulus);
    double             cur[24];
    for (int i = 0; i < 24; i++) cur[i] = X[i] + u[i];
    element.ComputeDeformationGradients(X, cur, F);
    nh.Stress(8, F, sigma);
    element.ComputeNodalForces(cur, sigma, f);
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  }
}

/* The reference neo-Hookean stress for n points (F [n][9] -> sigma [n][6]),
 * NeohookeanMaterial::GetStress (src/nimble_material.cc:252-310). */
int
nimref_stress(int n, const double* F, double bulk_modulus, double shear_modulus, double* sigma)
{
  try {
    MakeNeohookean(1.0, bulk_modulus, shear_modulus).Stress(n, F, sigma);
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  }
}

/* The reference's volume average of nq point quantities of one element,
 * HexElement::ComputeVolumeAverage (src/nimble_element.cc:262-282):
 * x_cur [8][3], q [8][nq] -> volume, avg [nq]. */
int
nimref_volume_average(const double* x_cur, int nq, const double* q, double* volume, double* avg)
{
  try {
    nimble::HexElement element;
    element.ComputeVolumeAverage(x_cur, nq, q, *volume, avg);
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  }
}

// A boundary-condition expression evaluated by the reference's own parser
// (ExpressionParsing::BoundaryConditionFunctor,
// src/nimble_expression_parser.h:697-800) at (x, y, z, t).
int
nimref_eval_expression(const char* text, double x, double y, double z, double t, double* value)
{
  try {
    ExpressionParsing::BoundaryConditionFunctor f{std::string(text)};
    *value = f.eval(x, y, z, t);
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  } catch (...) {
    g_last_error = "unknown exception";
    return -1;
  }
}

}  // extern "C"
