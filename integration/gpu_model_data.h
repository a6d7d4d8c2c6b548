// nimble::GpuModelData -- the reference-side adapter that puts the GB300
// engine (include/nimble_gb300.h, libnimble_gb300.so) behind NimbleSM's
// ModelData interface.
//
// NimbleSM's explicit loop (src/integrators/explicit_time_integrator.cc:177-278)
// sees only ModelDataBase virtuals (src/nimble_model_data_base.h:87-345).  This
// adapter subclasses the host nimble::ModelData (src/nimble_model_data.h), so
// the reference keeps its node storage, element-data labels, boundary
// conditions and output, and moves the element work to the GPU:
//   * InitializeBlocks: the reference's own block set-up, then one engine handle
//     over all blocks (blocks in increasing id, the order in which
//     ModelData::ComputeInternalForce visits them, src/nimble_model_data.cc:635-657);
//   * ComputeLumpedMass: the lumped mass and the critical time step
//     (src/nimble_model_data.cc:495-530, src/nimble_block_base.cc:51-84);
//   * ComputeInternalForce: u in, f_int out through the host-buffer entry point
//     (src/nimble_model_data.cc:620-667).  On output steps the deformation
//     gradient and Cauchy stress of every integration point are copied into the
//     reference's element data of step n+1, at the offsets
//     Block::ComputeInternalForce writes them to (src/nimble_block.cc:355-368,
//     labels from src/nimble_data_utils.cc:158-207), so that
//     WriteExodusOutput and ComputeDerivedElementData (src/nimble_block.cc:438-497)
//     read the stresses of the step.  The materials on this path keep no state
//     variables, and the reference reads element data only for output, so the
//     element data of other steps is not refreshed.
//
// Hook it in by changing the one line that creates the ModelData in
// DataManager::Initialize (src/nimble_data_manager.cc:113) to
// std::make_shared<nimble::GpuModelData>(), and link libnimble_gb300.so.
// The host-buffer call overlaps its copies with the element kernel only when
// the displacement and internal-force fields are page-locked: register them once
// after ModelData::Initialize allocates them (cudaHostRegister).
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nimble_data_manager.h"
#include "nimble_data_utils.h"
#include "nimble_genesis_mesh.h"
#include "nimble_material.h"
#include "nimble_model_data.h"
#include "nimble_gb300.h"

namespace nimble {

class GpuModelData : public ModelData
{
 public:
  ~GpuModelData() override
  {
    if (model_) nsm_destroy(model_);
  }

  // ModelData::InitializeBlocks (src/nimble_model_data.cc:484-493), then one
  // engine handle for all blocks: all nodes, the blocks' connectivity in
  // increasing block id and each block's material.
  void
  InitializeBlocks(DataManager& data_manager, const std::shared_ptr<MaterialFactoryBase>& factory) override
  {
    ModelData::InitializeBlocks(data_manager, factory);
    const GenesisMesh& mesh = data_manager.GetMesh();
    auto               X    = GetVectorNodeData("reference_coordinate");
    const int          N    = static_cast<int>(mesh.GetNumNodes());
    std::vector<double> xyz(3 * static_cast<size_t>(N));
    for (int n = 0; n < N; n++)
      for (int k = 0; k < 3; k++) xyz[3 * n + k] = X(n, k);
    std::vector<int>          conn, elem_block;
    std::vector<nsm_material> mats;
    blocks_in_order_.clear();
    for (auto& kv : GetBlocks()) {
      const int  block_id = kv.first;
      const int  ne       = mesh.GetNumElementsInBlock(block_id);
      const int* c        = mesh.GetConnectivity(block_id);
      conn.insert(conn.end(), c, c + 8 * static_cast<size_t>(ne));
      elem_block.insert(elem_block.end(), ne, static_cast<int>(mats.size()));
      const bool elastic = std::dynamic_pointer_cast<ElasticMaterial>(kv.second->GetMaterialPointer()) != nullptr;
      mats.push_back(nsm_material{elastic ? NSM_MATERIAL_ELASTIC : NSM_MATERIAL_NEOHOOKEAN, 0, kv.second->GetDensity(),
                                  kv.second->GetBulkModulus(), kv.second->GetShearModulus()});
      blocks_in_order_.push_back(BlockSpan{block_id, ne, {}, {}});
    }
    num_elem_ = static_cast<int>(elem_block.size());
    nsm_mesh_desc md{N, num_elem_, xyz.data(), conn.data()};
    nsm_options   opt{NSM_PRECISION_FP64, /*store_ip_data=*/1, /*device=*/0, /*graph_steps=*/0};
    Check(nsm_create_blocks(&md, static_cast<int>(mats.size()), elem_block.data(), mats.data(), &opt, &model_));
    FindElementDataOffsets();
  }

  // ModelData::ComputeLumpedMass (src/nimble_model_data.cc:495-530) and the
  // least critical time step over the blocks.
  void
  ComputeLumpedMass(DataManager& data_manager) override
  {
    auto mass = GetScalarNodeData("lumped_mass");
    Check(nsm_compute_lumped_mass(model_, mass.data()));
    double dt = 0.0;
    Check(nsm_critical_time_step(model_, &dt));
    SetCriticalTimeStep(dt);
  }

  // ModelData::ComputeInternalForce (src/nimble_model_data.cc:620-667).
  void
  ComputeInternalForce(
      DataManager&      data_manager,
      double            time_previous,
      double            time_current,
      bool              is_output_step,
      const Viewify<2>& displacement,
      Viewify<2>&       force) override
  {
    Check(nsm_compute_internal_force_host(model_, displacement.data(), force.data()));
    if (is_output_step) StoreElementData();
  }

 private:
  struct BlockSpan {
    int              block_id, num_elem;
    std::vector<int> def_grad_offset;  // [8 points x 9], the reference's K_F component order
    std::vector<int> stress_offset;    // [8 points x 6], K_S order
  };

  // The offsets of each point's deformation gradient and stress within a
  // block's per-element data, found by label as Block::DetermineDataOffsets
  // finds them (src/nimble_block.cc:500-545).
  void
  FindElementDataOffsets()
  {
    const auto& labels_of = GetElementDataLabels();
    for (BlockSpan& b : blocks_in_order_) {
      const std::vector<std::string>& labels = labels_of.at(b.block_id);
      auto find = [&](const std::string& label) {
        for (size_t i = 0; i < labels.size(); i++)
          if (labels[i] == label) return static_cast<int>(i);
        throw std::runtime_error("nimble_gb300: element data label " + label + " not declared");
      };
      b.def_grad_offset.clear();
      b.stress_offset.clear();
      for (int ip = 0; ip < 8; ip++) {
        for (int c = 0; c < 9; c++)
          b.def_grad_offset.push_back(find(GetComponentLabel("deformation_gradient", FULL_TENSOR, 3, c, ip + 1)));
        for (int c = 0; c < 6; c++)
          b.stress_offset.push_back(find(GetComponentLabel("stress", SYMMETRIC_TENSOR, 3, c, ip + 1)));
      }
    }
  }

  // F and sigma of the last force evaluation, [E][8][9] and [E][8][6] over the
  // handle's elements (blocks in increasing id), into each block's element
  // data of step n+1.
  void
  StoreElementData()
  {
    F_.resize(72 * static_cast<size_t>(num_elem_));
    sigma_.resize(48 * static_cast<size_t>(num_elem_));
    Check(nsm_get_ip_data(model_, F_.data(), sigma_.data()));
    size_t first = 0;  // the block's first element in the handle
    for (const BlockSpan& b : blocks_in_order_) {
      std::vector<double>& data = GetElementDataNew(b.block_id);
      const size_t         per  = b.num_elem > 0 ? data.size() / static_cast<size_t>(b.num_elem) : 0;
      for (size_t le = 0; le < static_cast<size_t>(b.num_elem); le++) {
        double*       dst = data.data() + le * per;
        const double* Fe  = F_.data() + 72 * (first + le);
        const double* Se  = sigma_.data() + 48 * (first + le);
        for (int j = 0; j < 72; j++) dst[b.def_grad_offset[j]] = Fe[j];
        for (int j = 0; j < 48; j++) dst[b.stress_offset[j]] = Se[j];
      }
      first += static_cast<size_t>(b.num_elem);
    }
  }

  static void
  Check(int status)
  {
    if (status != NSM_OK) throw std::runtime_error(std::string("nimble_gb300: ") + nsm_last_error());
  }

  nsm_model*             model_    = nullptr;
  int                    num_elem_ = 0;
  std::vector<BlockSpan> blocks_in_order_;
  std::vector<double>    F_, sigma_;
};

}  // namespace nimble
