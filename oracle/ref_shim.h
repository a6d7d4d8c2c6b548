/* Forced include for compiling the reference's host sources without Kokkos.
 *
 * TEST INFRASTRUCTURE ONLY (oracle). nimble_data_manager.cc:113 constructs
 * `nimble_kokkos::ModelData` unconditionally; without Kokkos that type does not
 * exist, so it is aliased here to the reference's own host `nimble::ModelData`
 * (nimble_model_data.h), which is what a non-Kokkos build of the explicit path
 * runs.  Nothing else in the reference is altered.
 */
#pragma once
namespace nimble { class ModelData; }
namespace nimble_kokkos { using ModelData = nimble::ModelData; }
