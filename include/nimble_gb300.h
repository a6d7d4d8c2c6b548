/* nimble_gb300 -- C ABI of the GB300 explicit-dynamics engine.
 *
 * The engine runs NimbleSM's explicit transient-dynamics step on one GPU:
 * 8-node hex elements with 2x2x2 Gauss points, neo-Hookean material, lumped
 * mass, central-difference time integration and velocity / displacement
 * boundary conditions.  These entry points are what a NimbleSM
 * ModelDataBase implementation (a "GpuModelData") forwards to: each one names
 * the reference interface it replaces (paths inside the NimbleSM source tree).
 *
 * Conventions
 *   - Plain C: opaque handles, host pointers and sizes, int status (0 = ok).
 *     On failure nsm_last_error() describes the error of the calling thread.
 *   - Host arrays use the reference layouts: node vectors [N][3] (x,y,z per
 *     node, src/nimble_model_data.cc:540-546), connectivity [E][8] 0-based in
 *     the reference corner order (src/nimble_element.cc:113-120), integration
 *     point tensors [E][8][9] full (K_F_* order xx,yy,zz,xy,yz,zx,yx,zy,xz)
 *     and [E][8][6] symmetric (K_S_* order xx,yy,zz,xy,yz,zx)
 *     (src/nimble_utils.h:91-109).
 *   - One handle = one block of elements on one GPU, one CUDA stream.  Calls on
 *     one handle must not overlap (like the reference's ModelData, which is not
 *     thread-safe); different handles are independent.
 *   - Arithmetic: NSM_PRECISION_FP64 computes in IEEE FP64 throughout.
 *     NSM_PRECISION_FP32_MIXED computes the element work (gradient, F, stress,
 *     B^T sigma) in FP32 and keeps the nodal state, mass, time step and
 *     energies in FP64.
 */
#ifndef NIMBLE_GB300_H
#define NIMBLE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSM_ABI_VERSION 1

/* Status codes. */
#define NSM_OK 0
#define NSM_ERR_INVALID_ARGUMENT 1
#define NSM_ERR_CUDA 2
#define NSM_ERR_BAD_JACOBIAN 3   /* an element inverted (det <= 0): the reference asserts, src/nimble_utils.h:1243-1255 */
#define NSM_ERR_NONFINITE 4      /* NaN/Inf in forces */
#define NSM_ERR_STATE 5          /* call out of order (e.g. advance before begin) */
#define NSM_ERR_OUT_OF_MEMORY 6

/* Precision forms. */
#define NSM_PRECISION_FP64 0
#define NSM_PRECISION_FP32_MIXED 1

/* Node fields (ModelData field labels, src/nimble_data_manager.cc:135-156). */
#define NSM_FIELD_REFERENCE_COORDINATE 0
#define NSM_FIELD_DISPLACEMENT 1
#define NSM_FIELD_VELOCITY 2
#define NSM_FIELD_ACCELERATION 3
#define NSM_FIELD_INTERNAL_FORCE 4
#define NSM_FIELD_EXTERNAL_FORCE 5   /* zero: ModelData::ComputeExternalForce zeroes it every step
                                        (src/nimble_model_data.cc:610-618), and a = (f_int + 0) / m */

/* Boundary-condition kinds (BoundaryCondition::BC_TYPE,
 * src/nimble_boundary_condition.h; parsed at src/nimble_boundary_condition.cc:65-144). */
#define NSM_BC_INITIAL_VELOCITY 0
#define NSM_BC_PRESCRIBED_VELOCITY 1
#define NSM_BC_PRESCRIBED_DISPLACEMENT 2

typedef struct nsm_model nsm_model;

typedef struct nsm_mesh_desc {
  int           num_nodes;
  int           num_elem;
  const double* coords; /* [N][3] reference coordinates */
  const int*    conn;   /* [E][8] */
} nsm_mesh_desc;

/* "neohookean density .. bulk_modulus .. shear_modulus .."
 * (NeohookeanMaterial, src/nimble_material.cc:208-224). */
typedef struct nsm_neohookean {
  double density;
  double bulk_modulus;
  double shear_modulus;
} nsm_neohookean;

/* A material of any supported model: the reference's material line
 * "<model> density .. bulk_modulus .. shear_modulus .." as MaterialFactory
 * creates it (src/nimble_material_factory.cc:57-70). */
#define NSM_MATERIAL_NEOHOOKEAN 0 /* NeohookeanMaterial, src/nimble_material.cc:208-310 */
#define NSM_MATERIAL_ELASTIC 1    /* ElasticMaterial (small strain on the unrotated F), src/nimble_material.cc:59-126 */
typedef struct nsm_material {
  int    model; /* NSM_MATERIAL_* */
  int    reserved;
  double density;
  double bulk_modulus;
  double shear_modulus;
} nsm_material;

typedef struct nsm_options {
  int precision;     /* NSM_PRECISION_* */
  int store_ip_data; /* 1: write F and sigma per integration point every step (the
                        ModelData element-data contract); 0: only on output steps */
  int device;        /* CUDA device ordinal */
  int graph_steps;   /* steps per captured CUDA graph in nsm_advance (0 = default 50) */
} nsm_options;

const char* nsm_last_error(void);
int         nsm_abi_version(void);

/* Mesh upload and one-time setup: reference geometry per integration point,
 * lumped mass and critical time step.  Replaces DataManager construction
 * (src/nimble_data_manager.cc:69-159) plus ModelData::InitializeBlocks
 * (src/nimble_model_data.cc:484-493) for one block. */
int nsm_create(const nsm_mesh_desc* mesh, const nsm_neohookean* material, const nsm_options* options,
               nsm_model** out);
int nsm_destroy(nsm_model* model);

/* Ensemble of independent samples in one handle (uncertainty quantification:
 * meshes of uneven size and per-sample material).  The samples' meshes are
 * concatenated: sample g's nodes and elements get global ids offset by
 * node_offsets[g] / elem_offsets[g] (nsm_ensemble_offsets), and every entry
 * point below works on the whole ensemble at once, each sample with its own
 * material and time schedule.  Each sample computes exactly what
 * nsm_create on its mesh alone computes.  The reference runs such samples one
 * at a time (one process per sample; its UQ mode, src/uq/nimble_uq_model_data.cc:145-248,
 * shares one mesh).  meshes, materials: [num_samples]. */
int nsm_create_ensemble(int num_samples, const nsm_mesh_desc* meshes, const nsm_neohookean* materials,
                        const nsm_options* options, nsm_model** out);

/* One mesh of several element blocks, each with its own material of any model
 * (ModelData::InitializeBlocks over all blocks, src/nimble_model_data.cc:484-493,
 * one Block and Material per "element block" line).  elem_block [E]: block
 * index 0..num_blocks-1 of each element, non-decreasing (the elements of a
 * block are contiguous, in the reference's block-by-block order, which is
 * also its assembly order); materials [num_blocks].  num_blocks = 1 with
 * elem_block NULL is a single block of any material model. */
int nsm_create_blocks(const nsm_mesh_desc* mesh, int num_blocks, const int* elem_block, const nsm_material* materials,
                      const nsm_options* options, nsm_model** out);

/* The reference's UQ mode on one mesh (nimble_uq::ModelData,
 * src/uq/nimble_uq_model_data.cc:145-248, with UqModel, src/uq/nimble_uq.cc):
 * trajectory 0 is the nominal (blocks and materials as nsm_create_blocks);
 * trajectories 1..num_exact evaluate the element forces with their own bulk
 * and shear moduli exact_bulk / exact_shear [num_exact][num_blocks]
 * (nimble_uq::Block::ComputeInternalForce, src/uq/nimble_uq_block.cc:57-164);
 * the last num_approx trajectories have no element work, their force being
 * the linear closure f = c_0 f_nominal + sum_k c_k f_exact_k with
 * coefficients [num_approx][num_exact + 1] (UqModel::ApplyClosure,
 * src/uq/nimble_uq.cc:327-345), and they use the nominal's lumped mass.  The
 * trajectories are samples of an ensemble (nsm_ensemble_offsets): give every
 * trajectory the velocity-type conditions and the nominal alone the
 * prescribed displacements (src/nimble_boundary_condition_manager.h:137-206),
 * and all of them the nominal's schedule (nsm_begin_ensemble). */
int nsm_create_uq(const nsm_mesh_desc* mesh, int num_blocks, const int* elem_block, const nsm_material* nominal,
                  int num_exact, const double* exact_bulk, const double* exact_shear, int num_approx,
                  const double* coefficients, const nsm_options* options, nsm_model** out);
int nsm_ensemble_offsets(nsm_model* model, int* node_offsets, int* elem_offsets); /* [S+1] each */
int nsm_ensemble_time_steps(nsm_model* model, double* dt);                      /* [S] critical steps */
/* Per-sample max |field component| over the listed (global) node ids, out [S]
 * (e.g. max |u_z| on each sample's top face). */
int nsm_ensemble_max_abs(nsm_model* model, int field, int component, const int* nodes, int count, double* out);

/* One boundary-condition line "<kind> <nodeset> <x|y|z> <value>" over a node
 * list, in deck order (BoundaryConditionManager::Initialize,
 * src/nimble_boundary_condition_manager.cc:52-72).  component 0..2. */
int nsm_add_boundary_condition(nsm_model* model, int kind, int component, double value, const int* nodes,
                               int num_nodes);
/* The same with the magnitude given by an expression f(x, y, z, t) (the
 * quoted form of a deck line, BoundaryCondition::Initialize,
 * src/nimble_boundary_condition.cc:102-117), evaluated at each node's
 * reference coordinates and at time_current whenever the condition is applied
 * (src/nimble_boundary_condition_manager.h:93-217).  The grammar is the
 * reference's ExpressionParsing (src/nimble_expression_parser.h:522-695):
 * + - * / % ^, unary -, ternary "c ? a : b" with | ^ & ! > >= < <= ==,
 * sin cos tan erf exp log abs asin acos atan sqrt cbrt erfc ceil round floor
 * log10, constants e pi tau.  NSM_ERR_INVALID_ARGUMENT with the parse error
 * when the text does not parse. */
int nsm_add_boundary_condition_expression(nsm_model* model, int kind, int component, const char* expression,
                                          const int* nodes, int num_nodes);
/* One host evaluation of an expression as the engine compiles it (the parse
 * and the operation order of the device evaluation, with the host's math
 * library), e.g. to check a deck's expressions before a run. */
int nsm_bc_expression_eval(const char* expression, double x, double y, double z, double t, double* value);

/* ModelData::ComputeLumpedMass (src/nimble_model_data.cc:495-530): the mass is
 * computed at nsm_create; this copies it out ([N], nullable). */
int nsm_compute_lumped_mass(nsm_model* model, double* lumped_mass);
/* ModelDataBase::GetCriticalTimeStep (src/nimble_model_data_base.h:297-300,
 * computed by src/nimble_block_base.cc:51-84). */
int nsm_critical_time_step(nsm_model* model, double* dt);

/* ModelDataBase::ApplyInitialConditions / ApplyKinematicConditions
 * (src/nimble_model_data_base.cc:83-100). */
int nsm_apply_initial_conditions(nsm_model* model);
int nsm_apply_kinematic_conditions(nsm_model* model, double time_current, double time_previous);

/* GetVectorNodeData views (src/nimble_model_data_base.h) as copies to / from
 * host [N][3] arrays. */
int nsm_set_node_field(nsm_model* model, int field, const double* values);
int nsm_get_node_field(nsm_model* model, int field, double* values);

/* ModelData::ComputeInternalForce (src/nimble_model_data.cc:620-667 ->
 * Block::ComputeInternalForce, src/nimble_block.cc:388-436) from the device
 * displacement into the device internal force; F_np1 and sigma_np1 are kept
 * per integration point. */
int nsm_compute_internal_force(nsm_model* model, double time_previous, double time_current, int is_output_step);

/* The same, with the displacement and the force in host memory: what the
 * reference's integrator loop (which updates nodes on the host) calls each
 * step through a GpuModelData.  displacement, internal_force: [N][3]. */
int nsm_compute_internal_force_host(nsm_model* model, const double* displacement, double* internal_force);
/* The reference integrator's loop on host arrays around the host-buffer call:
 * the step a NimbleSM run makes through the GpuModelData adapter, where
 * ExplicitTimeIntegrator keeps u, v, a in host memory
 * (src/integrators/explicit_time_integrator.cc:196-276: v += dt/2 a,
 * kinematic conditions, u += dt v, kinematic conditions,
 * nsm_compute_internal_force_host, a = f_int / m, v += dt/2 a, and the
 * kinematic conditions again on output steps).  num_steps steps from
 * *time_current with the user step dt_user (t += dt_user; the step's delta is
 * t - t_prev, as the reference forms it); step numbers first_step.. decide the
 * output steps (output_frequency, num_load_steps as in the input deck).
 * mass [N]; u, v, a, f_int [N][3] host arrays, updated in place; bcs (NULL:
 * none) the constant-magnitude conditions in deck order.  *host_seconds
 * (nullable) receives the time spent in the host-side updates.  The host
 * arithmetic rounds as the reference's, so the state equals nsm_advance's
 * bit for bit. */
typedef struct nsm_host_bcs {
  int           num_bcs;
  const int*    kind;      /* [num_bcs] NSM_BC_*; initial-velocity lines are skipped */
  const int*    component; /* [num_bcs] 0, 1, 2 */
  const double* value;     /* [num_bcs] */
  const int*    ptr;       /* [num_bcs + 1] offsets into nodes */
  const int*    nodes;
} nsm_host_bcs;
int nsm_host_loop_steps(nsm_model* model, int num_steps, double* time_current, double dt_user, int output_frequency,
                        int first_step, int num_load_steps, const double* mass, const nsm_host_bcs* bcs, double* u,
                        double* v, double* a, double* f_int, double* host_seconds);
/* The host-buffer call runs as a pipeline of `chunks` element ranges: u is
 * copied in by node ranges ahead of the element launches that need them and
 * f_int copied out by node ranges as soon as their elements are done, so the
 * copies overlap the element kernel (pinned buffers).  The result is bitwise
 * that of one launch.  0 restores the default (for 262,144 elements or
 * more 8 in FP64 and 4 in FP32, else 1); the learned and UQ closures always
 * run as one chunk. */
int nsm_set_host_chunks(nsm_model* model, int chunks);
int nsm_host_chunks(nsm_model* model, int* chunks);

/* Element data of the last internal-force evaluation, reference layout
 * (ModelData element data n/np1, src/nimble_model_data.cc:142-169).
 * F: [E][8][9], sigma: [E][8][6]; either may be NULL. */
int nsm_get_ip_data(nsm_model* model, double* F, double* sigma);

/* ---- block materials computed outside the engine (the plugin path) ----
 * The reference's BlockMaterialInterface (src/nimble_block_material_interface_base.h:52-84,
 * created by BlockMaterialInterfaceFactoryBase::create,
 * src/nimble_block_material_interface_factory_base.h:59-72) computes the stress of whole blocks on
 * the device between the kinematics and the stress divergence
 * (src/nimble_kokkos_model_data.cc:1180-1286), from F and sigma at steps n and n+1 and the
 * per-point state (Material::GetStress's device form, src/nimble_material.h:255-287).  With a
 * callback registered for a block, each step of the model runs the same split: the engine writes
 * F at n+1 of every point (and the built-in blocks' sigma), calls the callback of each such block
 * with device views of its points, then forms the nodal forces from the recorded sigma.  The
 * callback enqueues its own kernels on `stream` and returns 0 (nonzero: the step fails with
 * NSM_ERR_STATE); it must not synchronise the stream.  Record and state buffers of steps n and n+1
 * alternate after every step, as UpdateStates swaps the reference's element data.  A model with a
 * callback steps without CUDA graphs, so that the callback sees every step's times. */
typedef struct nsm_stress_request {
  int         block;                    /* block index, 0-based in the model's block order */
  int         elem_begin, elem_end;     /* the block's elements [begin, end) (blocks are contiguous) */
  int         precision;                /* NSM_PRECISION_FP64: double records, FP32_MIXED: float records */
  long        ld_e;                     /* record plane stride */
  const void* records_n;                /* step n:   [8 points][ld_e][16], F in slots 0..8 (K_F order), sigma 9..14 (K_S) */
  void*       records_np1;              /* step n+1: F written by the engine; the callback writes slots 9..14 */
  int         num_state;                /* state variables per point (as registered) */
  const double* state_n;                /* [8][ld_e][num_state] at step n, or NULL */
  double*       state_np1;              /* the same at n+1, written by the callback */
  double      time_n, time_np1;
  double      density, bulk_modulus, shear_modulus;  /* the block's material parameters */
  void*       stream;                   /* cudaStream_t */
} nsm_stress_request;
typedef int (*nsm_stress_callback)(void* user, const nsm_stress_request* request);
/* Registers `fn` for block `block` (replacing its built-in material) with num_state variables per
 * point (0 .. 64); NULL removes it.  Single-mesh models only (not ensembles or the UQ mode). */
int nsm_set_block_material_callback(nsm_model* model, int block, int num_state, nsm_stress_callback fn, void* user);
/* The per-point state after the last step, [E][8][num_state] (the largest registered count). */
int nsm_get_state_data(nsm_model* model, double* state);
/* Two callbacks written with the engine's own arithmetic, e.g. to check the path: the neo-Hookean
 * stress from F at n+1 (stateless), and the same with one history variable per point,
 * state_np1 = state_n + |det F_np1 - det F_n|. */
int nsm_example_neohookean_callback(void* user, const nsm_stress_request* request);
int nsm_example_history_callback(void* user, const nsm_stress_request* request);

/* Derived element output of the current configuration (replaces
 * Block::ComputeDerivedElementData, src/nimble_block.cc:438-497, through
 * HexElement::ComputeVolumeAverage, src/nimble_element.cc:262-282): element
 * volume [E], volume-averaged stress [E][6] and deformation gradient [E][9]
 * (reference component orders; weights det J of the current configuration
 * X + u), from the point data of the last evaluation that stored it.  Same
 * operations in the same order as the reference.  Any output may be NULL. */
int nsm_compute_derived_element_data(nsm_model* model, double* volume, double* stress, double* deformation_gradient);

/* Kinetic energy 1/2 sum m v.v and internal energy sum det(J_X) W(F) over the
 * integration points (not in the reference; used for energy balance). */
int nsm_get_energies(nsm_model* model, double* kinetic, double* internal);

/* The explicit loop of ExplicitTimeIntegrator::Integrate
 * (src/integrators/explicit_time_integrator.cc:123-278), on the device:
 * nsm_begin fixes the schedule (dt = (final - initial) / num_steps, output
 * steps every output_frequency and at the last step, 0 = none), zeroes the
 * state, applies the initial conditions, writes the optional initial velocity
 * v_init ([N][3], after ApplyInitialConditions) and applies the kinematic
 * conditions at t = 0.  nsm_advance runs the next num_steps steps of the
 * schedule as captured CUDA graphs; the state after each call is the
 * reference's state after that many steps. */
int nsm_begin(nsm_model* model, double initial_time, double final_time, int num_steps, int output_frequency,
              const double* v_init);
int nsm_advance(nsm_model* model, int num_steps);
/* nsm_begin for an ensemble: sample g runs num_steps steps of
 * dt_g = (final_times[g] - initial_time) / num_steps. */
int nsm_begin_ensemble(nsm_model* model, double initial_time, const double* final_times, int num_steps,
                       int output_frequency, const double* v_init);
/* nsm_advance bracketed by CUDA events on the handle's stream; waits for the
 * steps and returns their device time in milliseconds. */
int nsm_advance_timed(nsm_model* model, int num_steps, double* device_ms);
/* Steps done since nsm_begin and the current time. */
int nsm_progress(nsm_model* model, int* steps_done, double* time_current);
int nsm_synchronize(nsm_model* model);

/* Device status word accumulated since the last call (NSM_ERR_* mapped from
 * kernel-side checks: inverted elements, non-finite forces); clears it. */
int nsm_check_status(nsm_model* model);

/* Timing helpers for measurement: mean device time (CUDA events on the
 * handle's stream) of `repeats` launches of the element kernel alone and of
 * the node kernel alone, in milliseconds. */
int nsm_time_kernels(nsm_model* model, int repeats, double* element_ms, double* node_ms);
/* Picks the element kernel's launch shape (elements per block; one pass or a
 * persistent grid walking all samples' elements) by timing `repeats`
 * launches of each candidate on this model; returns the chosen candidate and
 * its mean time in milliseconds.  Captured graphs are rebuilt. */
int nsm_autotune(nsm_model* model, int repeats, int* chosen, double* best_ms);
/* The autotuner's measurements: mean milliseconds of `repeats` element-kernel
 * launches for each candidate launch shape, in candidate order, into
 * ms[0 .. capacity); *count receives the number of candidates.  The model's
 * own launch shape is left as it was. */
int nsm_launch_candidate_times(nsm_model* model, int repeats, double* ms, int capacity, int* count);
/* Sets the element kernel's launch shape to candidate `candidate` of the
 * autotuner's list (what nsm_autotune does with its choice). */
int nsm_set_launch_candidate(nsm_model* model, int candidate);
/* Number of kernel launches nsm_advance(model, num_steps) issues. */
int nsm_launches_per_advance(nsm_model* model, int num_steps);
/* Profiling mode: nsm_advance launches without CUDA graphs and brackets each
 * element and node kernel with CUDA events on the handle's stream;
 * nsm_get_profile returns (and resets) the summed device times and counts. */
int nsm_set_profiling(nsm_model* model, int enable);
int nsm_get_profile(nsm_model* model, double* element_ms_total, int* element_launches, double* node_ms_total,
                    int* node_launches);

/* Stable time step of the configuration X + u for a caller that cannot
 * allocate GPU memory (a framework that hands out all device buffers from its
 * own pool, code running during CUDA stream capture, a loop that must not
 * touch the allocator).  No counterpart in the reference: it is the reference's
 * GetCriticalTimeStep computation (min over elements of the characteristic
 * length over the bulk wave speed) without any allocation.  All pointers are
 * caller memory the GPU can read or write: coords [N][3], displacement [N][3]
 * (NULL = zero), conn [E][8], dt_out one double.  It runs on `stream` (a
 * cudaStream_t of the current device; NULL = the default stream) and returns
 * without waiting.  With no elements dt_out receives the largest double, as
 * nsm_critical_time_step gives for an empty model; a connectivity entry outside
 * [0, num_nodes) makes dt_out -1 (the element's coordinates are not read).
 * Its scratch is a fixed array inside this library sized for
 * NSM_NOALLOC_MAX_ELEMENTS elements (8 MiB per GPU, held until the process
 * exits); larger meshes are rejected with NSM_ERR_INVALID_ARGUMENT.  The first
 * call on a device looks up the array's device address and keeps it; make
 * that first call before any stream capture, and do not call it again on a
 * device after cudaDeviceReset (the kept address belongs to the old context).
 * Calls share the array: calls that overlap on the GPU (different streams or
 * threads) race and must be serialised by the caller.  Every error return
 * sets nsm_last_error(); a CUDA error left pending by the caller's earlier
 * work is reported as NSM_ERR_CUDA and not cleared. */
#define NSM_NOALLOC_MAX_ELEMENTS 1048576
int nsm_critical_time_step_noalloc(int num_nodes, int num_elem, const double* coords, const double* displacement,
                                   const int* conn, double density, double bulk_modulus, double* dt_out,
                                   void* stream);

/* ---- Learned constitutive closure ----
 * A 9 -> 64 -> 64 -> 6 MLP (GELU, BF16 weights, FP32 accumulation, trained
 * and evaluated on the 5th-generation tensor cores) that maps H = F - I to
 * the Cauchy stress over the shear modulus, standing in for the neo-Hookean
 * material update behind the same material interface (the reference's
 * Material::GetStress, src/nimble_material.h:239-313; no learned material
 * exists in the reference).  It is placed on the material's second-order
 * expansion with a cubic gate: sigma/G = B(H) + s_r |x|^3 MLP(x),
 * x = H * in_scale, B the neo-Hookean stress to second order in H, so the
 * network carries the O(|H|^3) remainder and cannot disturb the response
 * near F = I, where its training data is thinnest.  Points outside the
 * training envelope (|H_ij| > 4 s_in^-1 or det F < min_det) use the plain
 * neo-Hookean stress.  Parameters: W1[64][9], b1[64], W2[64][64], b2[64],
 * W3[6][64], b3[6] (NSM_MLP_PARAMS floats); scales: in_scale, res_scale,
 * K/G, envelope, min_det. */
#define NSM_MLP_PARAMS 5190
typedef struct nsm_mlp nsm_mlp;
const char* nsm_mlp_last_error(void);
int nsm_mlp_create(double bulk_modulus, double shear_modulus, unsigned long long seed, int device, nsm_mlp** out);
int nsm_mlp_destroy(nsm_mlp* mlp);
/* Training set on the device: n pairs F = I + N(0, perturbation^2) per entry,
 * det F >= min_det (rejection), sigma from the neo-Hookean material. */
int nsm_mlp_generate(nsm_mlp* mlp, long n, unsigned long long seed, double perturbation, double min_det);
/* Adam on the mean squared error of the scaled residual, minibatches of
 * 128 * batch_tiles points, cosine learning-rate decay; returns the last
 * epoch's mean loss per output component. */
int nsm_mlp_train(nsm_mlp* mlp, int epochs, int batch_tiles, double lr, double* final_loss);
int nsm_mlp_get_params(nsm_mlp* mlp, float* params, float* scales);
/* Copy of training pairs [first, first + count): H [count][9], sigma/G [count][6]. */
int nsm_mlp_training_sample(nsm_mlp* mlp, long first, long count, float* H, float* Y);
int nsm_mlp_set_params(nsm_mlp* mlp, const float* params, const float* scales);
/* Gradient of the training loss over n given pairs (H row-major [n][9],
 * sigma/G [n][6]) with respect to the parameters, as the training kernel
 * computes it; loss = mean over points of the squared scaled residual. */
int nsm_mlp_gradient(nsm_mlp* mlp, long n, const float* H, const float* Y, float* grad, double* loss);
/* Stress of n deformation gradients (reference slot order [n][9]) -> sigma
 * [n][6]; fallback_count = points outside the envelope (plain material). */
int nsm_mlp_predict(nsm_mlp* mlp, long n, const double* F, double* sigma, int* fallback_count);

/* Use the learned closure as the material of a model's element kernel (the
 * FP32-mixed form, one material; NULL restores the neo-Hookean stress).  The
 * closure's parameters are read at every launch, so training may continue
 * between steps.  nsm_closure_fallbacks: integration-point evaluations that
 * left the training envelope and used the plain material, since the model
 * was created. */
int nsm_set_mlp_closure(nsm_model* model, nsm_mlp* closure);
int nsm_closure_fallbacks(nsm_model* model, unsigned long long* count);

/* Diagnostic: D[128][N] = A[128][K] * B[N][K]^T on the 5th-generation
 * tensor cores (operands rounded to BF16, FP32 accumulation), through the
 * same primitives and shared-memory layout as the learned closure's kernels.
 * N, K multiples of 16, N <= 256, K <= 128; host arrays. */
int nsm_tc_selftest(int N, int K, const float* A, const float* B, float* D);

/* Diagnostic of the failure path of the tensor-core waits: a kernel that
 * holds tensor memory waits on an mbarrier phase that nothing completes,
 * bounded by `limit_us` (1..100000) microseconds of GPU time; *timed_out = 1
 * when the wait ran out, after which the kernel freed its tensor memory and
 * returned.  The context stays usable.  (Every tensor-core wait of the
 * library is bounded the same way, at one second.) */
int nsm_tc_wait_timeout_selftest(long limit_us, int* timed_out);

/* Number of SMs of the device. */
int nsm_device_sm_count(int device, int* count);

/* Pinned host memory for the host-buffer entry points (page-locked so that the
 * copies run at full link bandwidth). */
void* nsm_host_alloc(size_t bytes);
void  nsm_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif
