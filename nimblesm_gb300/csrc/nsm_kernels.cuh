// Kernel launch interfaces of the engine (device layouts are structure of
// arrays: a node field of 3 components is three planes of ld_n doubles; an
// element field is planes of ld_e entries, one plane per component).
#pragma once

#include <string>
#include <vector>

#include "nsm_common.cuh"

// Device status word bits (read back by the host, returned as C status codes).
#define NSM_STATUS_BAD_JACOBIAN 1   // a non-positive Jacobian determinant (inverted element)
#define NSM_STATUS_NONFINITE 2      // a NaN or Inf in a stress or force
#define NSM_STATUS_TIMEOUT 8        // a bounded wait on the tensor cores ran out

struct nsm_model;  // the handle of include/nimble_gb300.h

namespace nsm {

// One material: of a block of a multi-block mesh, or of one sample of an
// ensemble (one entry for a single mesh).
struct GroupMaterial {
  double bulk, shear, density, sound_speed;
  int    model;
  int    pad;
};

// Reference geometry per integration point (FP64 form), planes
// [8 * kGeoPerPoint][ld_e]: per point J_X^{-1} / 8 (9, row-major), det J_X,
// 8 J_X = 8 dX/dxi (9, row-major) and 1 / (512 det J_X).  The factors are
// those of the modal gradient (8 du/dxi); powers of two, so exact.
constexpr int kGeoPerPoint = 20;

struct SetupArgs {
  int           N, E;
  int           num_groups;      // samples; elements of sample g are [elem_off[g], elem_off[g+1])
  const int*    elem_group;      // [E] material of each element (null: material 0)
  const int*    elem_off;        // [num_groups+1]
  const GroupMaterial* mats;     // materials
  long          ld_n, ld_e;
  const int*    conn;      // [8][ld_e]
  const double* X;         // [3][ld_n]
  const int*    node_ptr;  // [N+1]
  const int*    node_inc;  // 8*e + corner, increasing e per node
  double*       geo;       // [8 * kGeoPerPoint][ld_e]
  double*       me;        // [8][ld_e]
  double*       dt_elem;   // [E]
  double*       dt_partial;// [1024]
  double*       dt_out;    // [num_groups] per-sample critical time step
  double*       mass;      // [N]
  double*       inv_mass;  // [N]
  int*          status;
};

void        shape_tables(double* N, double* dN);
cudaError_t upload_shape_tables(cudaStream_t stream);
cudaError_t launch_setup(const SetupArgs& a, cudaStream_t stream);
// Element volume [E], volume-averaged stress [E][6] and deformation
// gradient [E][9] of the current configuration from the point records
// (setup_kernels.cu).
cudaError_t launch_derived_element(int E, long ld_e, const int* conn, const double* X, const double* u, long ld_n,
                                   const void* ip, int ip_is_float, double* volume, double* avg_sigma, double* avg_F,
                                   int* status, cudaStream_t stream);

// Per-point record of the element data: 16 values of type T per element and
// integration point, records laid out [ip][ld_e][16]: slots 0..8 F in the
// reference full-tensor order, 9..14 sigma in the symmetric order, 15 unused.
// One thread writes its 64 (FP32) or 128 (FP64) contiguous bytes with vector
// stores; a warp writes 2 or 4 KB contiguous.
constexpr int kIpRecord = 16;

// Element kernel arguments (one launch = all elements of a block).
struct ElementArgs {
  int           E;         // elements [e_begin, E) are computed by this launch
  int           e_begin;
  long          ld_e, ld_n;
  const int*    conn;      // [8][ld_e]
  const double* u;         // [3][ld_n] displacement (FP64 form)
  const float*  uf;        // [3][ld_n] FP32 copy of u (FP32 form)
  const float*  Xf;        // [3][ld_n] FP32 copy of X (FP32 form)
  const double* geo;       // [8 * kGeoPerPoint][ld_e] (FP64 form only)
  double        bulk, shear;     // material when elem_group is null
  int           model;           // material model when elem_group is null
  const int*    elem_group;      // [E] material of each element, or null
  const GroupMaterial* mats;     // materials
  int           num_groups;      // samples (rows of the schedule)
  int           persistent;      // 0: one thread per element; 1: grid-stride over elements
  void*         ip;        // [8][ld_e][16] per-point records (T)
  void*         fe;        // [ld_e][24] element nodal forces, corner-major (T)
  int               store_ip;   // 1: write F and sigma; 0: only on output steps of the schedule
  const StepSched*  sched;      // schedule (nullable: outside the time loop)
  const int*        step_base;  // device step counter
  int               k;          // schedule offset of this step
  int*              status;
};

// Launch shape of the element kernel (chosen by the autotuner).
struct ElementLaunch {
  int block;        // threads per block
  int persistent;   // 0: one thread per element, 1: grid-stride with `waves` blocks per SM
  int blocks_per_sm;
  int staged;       // FP32 form: persistent, nodal values staged one element ahead by cp.async
};
cudaError_t launch_element_fp64(const ElementArgs& a, const ElementLaunch& l, cudaStream_t stream);
cudaError_t launch_element_fp32(const ElementArgs& a, const ElementLaunch& l, cudaStream_t stream);
// The split step of models with a block-material callback: pass 1 the
// kinematics (F, built-in sigma, records), pass 2 the forces from the
// recorded sigma (one thread per element).
cudaError_t launch_element_pass(const ElementArgs& a, int is_float, int pass, cudaStream_t stream);
int         num_sms();
// F = I (sigma = 0) in every point record: the element data before the first step.
cudaError_t launch_ip_identity(int E, long ld_e, void* ip, int ip_is_float, cudaStream_t stream);

// Node kernel: the end of step s (gather f_int, a = f/m, v += half*a, output
// BCs) fused with the start of step s+1 (v += half*a, BCs, u += delta*v, BCs).
// The expression programs of a model's boundary conditions and the node
// coordinates they read (x, y, z of the reference configuration).
struct BcExprTable {
  const ExprOp* code;   // programs, concatenated
  const int*    start;  // [programs + 1] first op of each
  const double* X;      // [3][ld_n]
  long          ld_n;
};

// Boundary-condition expressions (bc_expression.cu): the reference's grammar
// to a postfix program appended to `code` (an error message, or empty); one
// operation and a whole program evaluated on the host.
std::string compile_bc_expression(const std::string& text, std::vector<ExprOp>& code);
double      apply_host(int code, double a, double b);
double      eval_bc_expression_host(const ExprOp* code, int count, double x, double y, double z, double t);

struct NodeArgs {
  int               N;        // nodes [n_begin, N) are updated by this launch
  int               n_begin;
  long              ld_n, ld_e;
  const int*        node_ptr;
  const int*        node_inc;
  // the first 8 incidences of each node, slot-major [8][ld_n] (-1 past the
  // node's last), and a bit per node set when it has more (read from node_inc)
  const int*        node_slots;
  const unsigned*   node_more;
  const void*       fe;       // element nodal forces (double or float)
  int               fe_is_float;
  const double*     inv_mass;
  const int*        bc_slot;  // [N] -1 or index into bcs
  const NodeBC*     bcs;
  const StepSched*  sched;    // per-step schedule [step][num_groups]
  const int*        step_base;// device step counter (schedule index of step "k = 0")
  const int*        node_group; // [N] sample of each node, or null
  int               num_groups;
  int               k_post;   // schedule offset of the step being finished, or -1
  int               k_pre;    // schedule offset of the step being started, or -1
  int               gather_only; // only f_int = gather(fe); no state update
  double*           u;
  double*           v;
  double*           a;
  double*           f_int;
  float*            uf;       // FP32 copy of u kept in step (FP32 form), or null
  // UQ closure (samples of one mesh): samples closure_first.. have no
  // elements; their force is c0 f_0 + sum_k c_k f_k over samples 0..num_exact
  // at the same local node (closure [sample - closure_first][num_exact + 1]).
  const double*     closure;  // or null
  int               closure_first, num_exact;
  const int*        node_off; // [num_groups + 1] first node of each sample
  // expression-driven boundary conditions: their values for this launch,
  // [2][num_bc_slots][3] (level 0 at the step finished, 1 at the step
  // started; launch_bc_expr_values), or null when no condition has one
  const double*     bc_expr_val;
  int               num_bc_slots;
};

cudaError_t launch_node_update(const NodeArgs& a, cudaStream_t stream);
// The values a.bc_expr_val holds for the node launch of `a` (k_post, k_pre):
// each kinematic slot's expressions at its node (slot_node) and at the
// schedule's time of those steps.
cudaError_t launch_bc_expr_values(const NodeArgs& a, const int* slot_node, const BcExprTable& ex,
                                  double* out, cudaStream_t stream);
cudaError_t launch_advance_base(int* step_base, int k, cudaStream_t stream);

// Kinematic conditions alone (ApplyKinematicConditions with delta_t), and
// initial conditions (velocity values).
cudaError_t launch_apply_bc(int N, long ld_n, const int* bc_slot, const NodeBC* bcs, double delta, double time,
                            const BcExprTable& ex, const double* u, double* v, cudaStream_t stream);

// Energies: kinetic 1/2 m v.v (per-node) and internal sum det J0 W(F) per ip;
// two-pass deterministic sums into out[0], out[1].
constexpr int kEnergyBlocks = 608;  // 4 x 152 SMs; partial buffer holds 2 doubles per block
cudaError_t   launch_energies(int N, long ld_n, const double* mass, const double* v, int E, long ld_e,
                              const int* conn, const double* u, const double* geo, const int* elem_group,
                              const GroupMaterial* mats, double* partial, double* out, cudaStream_t stream);

// Per-sample max |field_c| over listed nodes (node ids global; sample from
// node_group, or sample 0).  out: [num_groups], zeroed by the launcher.
cudaError_t launch_group_max_abs(int count, const int* nodes, const double* field, long ld_n, int component,
                                 const int* node_group, int num_groups, double* out, cudaStream_t stream);

// Reference-layout views of SoA data ([E][8][9] / [E][8][6] / [N][3]).
// which: 0 = F ([E][8][9]), 1 = sigma ([E][8][6]).
cudaError_t launch_ip_to_aos(int E, long ld_e, const void* ip, int src_is_float, int which, double* dst,
                             cudaStream_t stream);
cudaError_t launch_to_float(long n, const double* src, float* dst, cudaStream_t stream);
cudaError_t launch_node_soa_to_aos(int N, long ld_n, const double* src, double* dst, cudaStream_t stream);
// dstf (nullable): also an FP32 copy of the planes, same layout.
cudaError_t launch_node_aos_to_soa(int N, long ld_n, const double* src, double* dst, float* dstf,
                                   cudaStream_t stream);

// Records the calling thread's nsm_last_error() text and returns `code`
// (for entry points defined outside nsm_model.cu).
int set_last_error(int code, const char* msg);
// Number of nodes of a handle (all samples of an ensemble).
int model_num_nodes(const ::nsm_model* m);

}  // namespace nsm
