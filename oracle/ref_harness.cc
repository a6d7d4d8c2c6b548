/* Reference harness: drives NimbleSM's own host objects (compiled from the
 * reference sources by oracle/Makefile) on an in-memory mesh.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product: it
 * is linked only into oracle/_ref/libnimble_ref.so and is loaded only by the
 * tests, by tests/golden/make_golden.py and by the CPU-baseline leg of
 * bench.py.
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
#include "nimble_genesis_mesh.h"
#include "nimble_material.h"
#include "nimble_material_factory.h"
#include "nimble_model_data.h"
#include "nimble_parser.h"
#include "nimble_view.h"

namespace {

// Fills the protected members of the reference's mesh class
// (src/nimble_genesis_mesh.h:328-354) directly, as ReadTextFile does
// (src/nimble_genesis_mesh.cc:318-427), but from memory: one block with id 1.
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
      const std::vector<std::string>& ns_names)
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
    block_ids_                   = {1};
    all_block_ids_               = {1};
    block_names_[1]              = "block_1";
    all_block_names_[1]          = "block_1";
    block_elem_global_ids_[1]    = elem_global_id_;
    block_num_nodes_per_elem_[1] = 8;
    block_elem_connectivity_[1]  = std::vector<int>(conn, conn + 8 * static_cast<size_t>(num_elem));
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
 * xyz[3N], conn[8E] (0-based, reference corner order), node sets in CSR form
 * (ns_ptr[num_node_sets+1], ns_nodes) with '\n'-separated names, the material
 * line as in an input deck ("neohookean density .. bulk_modulus .. shear_modulus .."),
 * '\n'-separated boundary-condition lines.  v_init (nullable, [N][3]) is
 * written into the velocity after ApplyInitialConditions and before
 * ApplyKinematicConditions(0,0).  Outputs: u, v, a, f_int [N][3]; F [E][8][9]
 * and sigma [E][8][6] in the reference component order (nullable); lumped
 * mass [N]; critical time step; wall seconds of the step loop.
 * Returns 0, or -1 with nimref_last_error() set. */
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
  try {
    HarnessMesh mesh;
    mesh.Fill(num_nodes, xyz, num_elem, conn, num_node_sets, ns_ptr, ns_nodes, SplitLines(ns_names));

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
    parser.Set("material parameters", std::string("material_1 ") + material);
    parser.Set("element block", "block_1 material_1");
    parser.Set("output fields", "displacement");
    for (auto const& bc : SplitLines(bcs)) parser.Set("boundary condition", bc);

    nimble::DataManager data_manager(parser, mesh);
    auto                model_data_ptr = data_manager.GetModelData();
    auto&               model_data     = *model_data_ptr;
    model_data.InitializeBlocks(data_manager, std::make_shared<nimble::MaterialFactory>());

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

    model_data.ApplyInitialConditions(data_manager);
    if (v_init != nullptr) {
      for (int i = 0; i < num_nodes; i++)
        for (int k = 0; k < 3; k++) velocity(i, k) = v_init[3 * i + k];
    }
    model_data.ApplyKinematicConditions(data_manager, 0.0, 0.0);

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
    }
    auto t1 = std::chrono::steady_clock::now();

    if (out_loop_seconds) *out_loop_seconds = std::chrono::duration<double>(t1 - t0).count();
    if (out_dt_crit) *out_dt_crit = critical_time_step;
    for (int i = 0; i < num_nodes; i++) {
      for (int k = 0; k < 3; k++) {
        if (out_u) out_u[3 * i + k] = displacement(i, k);
        if (out_v) out_v[3 * i + k] = velocity(i, k);
        if (out_a) out_a[3 * i + k] = acceleration(i, k);
        if (out_fint) out_fint[3 * i + k] = internal_force(i, k);
      }
      if (out_mass) out_mass[i] = lumped_mass(i);
    }

    // Per-integration-point F and sigma of the last internal-force evaluation:
    // re-evaluated from the final displacement with the reference's own
    // element and material (the same calls the block functor makes,
    // src/nimble_block.cc:309-352), which reproduces the stored values exactly.
    if (out_F || out_sigma) {
      nimble::HexElement element;
      auto               block    = std::dynamic_pointer_cast<nimble::ModelData>(model_data_ptr)->GetBlocks().at(1);
      auto               nh       = MakeNeohookean(block->GetDensity(), block->GetBulkModulus(), block->GetShearModulus());
      double             ref_coord[24], cur_coord[24], F[72], sig[48];
      for (int e = 0; e < num_elem; e++) {
        for (int n = 0; n < 8; n++) {
          int id = conn[8 * e + n];
          for (int k = 0; k < 3; k++) {
            ref_coord[3 * n + k] = xyz[3 * id + k];
            cur_coord[3 * n + k] = xyz[3 * id + k] + displacement(id, k);
          }
        }
        element.ComputeDeformationGradients(ref_coord, cur_coord, F);
        nh.Stress(8, F, sig);
        if (out_F) std::memcpy(out_F + 72 * static_cast<size_t>(e), F, sizeof(F));
        if (out_sigma) std::memcpy(out_sigma + 48 * static_cast<size_t>(e), sig, sizeof(sig));
      }
    }
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  }
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

/* The reference's volume average of one element's point stresses,
 * HexElement::ComputeVolumeAverage (src/nimble_element.cc:262-282):
 * x_cur [8][3], sigma [8][6] -> volume, avg [6]. */
int
nimref_volume_average(const double* x_cur, const double* sigma, double* volume, double* avg)
{
  try {
    nimble::HexElement element;
    element.ComputeVolumeAverage(x_cur, 6, sigma, *volume, avg);
    return 0;
  } catch (std::exception const& ex) {
    g_last_error = ex.what();
    return -1;
  }
}

}  // extern "C"
