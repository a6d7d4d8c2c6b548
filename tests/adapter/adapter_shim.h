/* Forced include for the adapter test (TEST INFRASTRUCTURE ONLY): the
 * reference's DataManager::Initialize (src/nimble_data_manager.cc:113)
 * creates `nimble_kokkos::ModelData`; aliasing that name to the adapter is the
 * one-line hook a maintainer makes in the reference, so the reference's own
 * DataManager builds a nimble::GpuModelData. */
#pragma once
#include "gpu_model_data.h"
namespace nimble_kokkos { using ModelData = nimble::GpuModelData; }
