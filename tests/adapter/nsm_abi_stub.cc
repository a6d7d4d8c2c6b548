// TEST-ONLY stand-in for the engine's C ABI (include/nimble_gb300.h), built on
// the CPU oracle (oracle/nsm_oracle.c), so that the reference-side adapter
// (integration/gpu_model_data.h) can be driven by the reference's own
// DataManager and explicit loop on a machine without a GPU.  Only the calls the
// adapter makes are provided.  It is compiled and loaded by
// tests/test_integration_adapter.py alone and is never part of the engine
// library (nimblesm_gb300/).
#include <cstring>
#include <string>
#include <vector>

#include "nimble_gb300.h"
#include "nsm_oracle.h"

struct nsm_model {
  std::vector<double> coords;
  std::vector<int>    conn, elem_block, block_model;
  std::vector<double> block_density, block_bulk, block_shear;
  nsm_oracle_model    m{};
  nsm_oracle*         o = nullptr;
};

namespace {
thread_local std::string g_error;
int fail(int code, const char* msg)
{
  g_error = msg;
  return code;
}
}  // namespace

extern "C" {

const char* nsm_last_error(void) { return g_error.c_str(); }

int nsm_create_blocks(const nsm_mesh_desc* mesh, int num_blocks, const int* elem_block, const nsm_material* materials,
                      const nsm_options* opt, nsm_model** out)
{
  if (!mesh || !materials || !out || num_blocks < 1) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  if (opt && opt->precision != NSM_PRECISION_FP64) return fail(NSM_ERR_INVALID_ARGUMENT, "stub: FP64 only");
  nsm_model* h = new nsm_model;
  const int  N = mesh->num_nodes, E = mesh->num_elem;
  h->coords.assign(mesh->coords, mesh->coords + 3 * static_cast<size_t>(N));
  h->conn.assign(mesh->conn, mesh->conn + 8 * static_cast<size_t>(E));
  h->elem_block.assign(E, 0);
  if (elem_block) h->elem_block.assign(elem_block, elem_block + E);
  for (int b = 0; b < num_blocks; b++) {
    h->block_model.push_back(materials[b].model == NSM_MATERIAL_ELASTIC ? NSM_ORACLE_ELASTIC : NSM_ORACLE_NEOHOOKEAN);
    h->block_density.push_back(materials[b].density);
    h->block_bulk.push_back(materials[b].bulk_modulus);
    h->block_shear.push_back(materials[b].shear_modulus);
  }
  nsm_oracle_model& m = h->m;
  m.num_nodes         = N;
  m.num_elem          = E;
  m.coords            = h->coords.data();
  m.conn              = h->conn.data();
  m.density           = materials[0].density;
  m.bulk_modulus      = materials[0].bulk_modulus;
  m.shear_modulus     = materials[0].shear_modulus;
  m.material_model    = h->block_model[0];
  m.num_blocks        = num_blocks;
  m.elem_block        = h->elem_block.data();
  m.block_model       = h->block_model.data();
  m.block_density     = h->block_density.data();
  m.block_bulk        = h->block_bulk.data();
  m.block_shear       = h->block_shear.data();
  h->o                = nsm_oracle_create(&h->m, 1);
  if (!h->o) {
    delete h;
    return fail(NSM_ERR_OUT_OF_MEMORY, "oracle allocation failed");
  }
  *out = h;
  return NSM_OK;
}

int nsm_destroy(nsm_model* h)
{
  if (h) {
    nsm_oracle_destroy(h->o);
    delete h;
  }
  return NSM_OK;
}

int nsm_compute_lumped_mass(nsm_model* h, double* mass)
{
  if (!h || !mass) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  nsm_oracle_get_state(h->o, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, mass);
  return NSM_OK;
}

int nsm_critical_time_step(nsm_model* h, double* dt)
{
  if (!h || !dt) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  *dt = nsm_oracle_dt_crit(h->o);
  return NSM_OK;
}

int nsm_compute_internal_force_host(nsm_model* h, const double* u, double* f)
{
  if (!h || !u || !f) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  return nsm_oracle_internal_force(h->o, u, f) == 0 ? NSM_OK
                                                   : fail(NSM_ERR_BAD_JACOBIAN, "non-positive Jacobian");
}

int nsm_get_ip_data(nsm_model* h, double* F, double* sigma)
{
  if (!h) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  nsm_oracle_get_state(h->o, nullptr, nullptr, nullptr, nullptr, F, sigma, nullptr);
  return NSM_OK;
}

}  // extern "C"
