// Host engine of the C ABI (include/nimble_gb300.h): device-resident
// ModelData for one block, the explicit loop as captured CUDA graphs, and the
// host-buffer entry points.  C++ host code; all arithmetic on the path runs
// in the kernels (setup_kernels.cu, element_kernels.cu, node_kernels.cu).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "../../include/nimble_gb300.h"
#include "mlp_element.cuh"
#include "nsm_kernels.cuh"

using nsm::NodeBC;
using nsm::StepSched;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg)
{
  g_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where)
{
  g_error = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? NSM_ERR_OUT_OF_MEMORY : NSM_ERR_CUDA;
}

#define NSM_CUDA(call)                                    \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);   \
  } while (0)

long pad(long n, long q) { return (n + q - 1) / q * q; }

struct BcLine {
  int              kind, component;
  double           value;
  std::vector<int> nodes;
  int              expr = -1;  // expression program giving the value, or -1
};

}  // namespace

struct nsm_model {
  int          N = 0, E = 0, S = 1;  // nodes, elements, samples
  std::vector<int> node_off, elem_off;  // per-sample offsets [S+1]
  long         ld_n = 0, ld_e = 0;
  int          precision = NSM_PRECISION_FP64, store_ip = 1, graph_steps = 50, device = 0;
  double       density = 0, K = 0, G = 0, dt_crit = 0;  // material 0
  int          model = NSM_MATERIAL_NEOHOOKEAN, num_mats = 1;
  cudaStream_t stream = nullptr;

  int*    d_conn = nullptr;  // [8][ld_e]
  int*    d_node_ptr = nullptr;
  int*    d_node_inc = nullptr;
  int*      d_node_slots = nullptr;  // [8][ld_n] first 8 incidences of each node, -1 past its last
  unsigned* d_node_more  = nullptr;  // bit n: node n has more than 8 incidences
  double* d_X = nullptr;  // node planes [3][ld_n]
  double* d_u = nullptr;
  double* d_v = nullptr;
  double* d_a = nullptr;
  double* d_f = nullptr;
  double* d_fext = nullptr;
  double* d_mass = nullptr;
  double* d_inv_mass = nullptr;
  double* d_geo = nullptr;  // [8 * kGeoPerPoint][ld_e]
  void*   d_ip = nullptr;   // [8][ld_e][16] per-point F and sigma records
  void*   d_fe = nullptr;   // [24][ld_e] element nodal forces, corner-major planes (3 c + i)
  float*  d_Xf = nullptr;   // FP32 copies of X and u (FP32 form)
  float*  d_uf = nullptr;
  int*    d_status = nullptr;
  int*    d_step_base = nullptr;
  double* d_scratch = nullptr;  // energy partials / setup temporaries
  double* d_stage = nullptr;    // [3N] AoS staging for host copies
  double* d_out = nullptr;      // small results
  double* d_group_out = nullptr;// [S] per-sample results
  int*    d_elem_group = nullptr;  // [E] material of each element (more than one material)
  int*    d_node_group = nullptr;  // [N] sample of each node (S > 1)
  int*    d_elem_off = nullptr;    // [S+1]
  int*    d_node_off = nullptr;    // [S+1] (UQ closure)
  double* d_closure = nullptr;     // [num_approx][num_exact+1] (UQ closure), or null
  int     closure_first = 0, num_exact = 0;
  nsm::GroupMaterial* d_mats = nullptr;  // [num_mats]
  std::vector<double> dt_group;    // per-sample critical time step
  nsm::ElementLaunch  elaunch{128, 0, 0, 0};
  nsm_mlp*            closure = nullptr;        // learned material (FP32 form), or null
  // block materials computed by callbacks (the plugin path)
  struct BlockCallback {
    nsm_stress_callback fn = nullptr;
    void*               user = nullptr;
    int                 num_state = 0;
  };
  std::vector<BlockCallback>       block_cb;       // per block (material index)
  std::vector<nsm::GroupMaterial>  h_mats;         // host copy of the materials, as created
  std::vector<std::pair<int, int>> block_range;    // elements [first, last) of each block
  int                              num_state = 0;  // per point, the largest registered
  void*                            d_ip_n = nullptr;     // records of step n (the split step)
  double*                          d_state = nullptr;    // [8][ld_e][num_state], latest
  double*                          d_state_n = nullptr;  // the step before
  double                           ci_t_prev = 0, ci_t_cur = 0;  // times of a direct internal-force call
  bool                             cb_failed = false;            // a callback returned nonzero
  float*              d_closure_geo = nullptr;  // [ld_e][8][12] its reference geometry per point
  unsigned long long* d_fallbacks = nullptr;    // points that left the closure's envelope

  std::vector<BcLine> bcs;
  bool                bcs_dirty = true;
  std::vector<nsm::ExprOp> expr_code;           // expression programs, concatenated
  std::vector<int>         expr_start{0};       // [programs + 1]
  nsm::ExprOp*             d_expr_code = nullptr;
  int*                     d_expr_start = nullptr;
  int                      num_bc_slots = 0;          // nodes with a kinematic condition
  int*                     d_bc_slot_node = nullptr;  // [num_bc_slots] their node ids
  bool                     bc_has_expr = false;       // some kinematic condition is an expression
  double*                  d_bc_expr_val = nullptr;   // [2][num_bc_slots][3] values per node launch
  int*                d_bc_slot = nullptr;
  NodeBC*             d_bcs = nullptr;
  int*                d_ibc_slot = nullptr;
  NodeBC*             d_ibcs = nullptr;

  // schedule
  bool                   begun = false;
  int                    num_steps = 0, steps_done = 0;
  std::vector<StepSched> h_sched;
  std::vector<double>    h_time;  // time after each step
  double                 t0 = 0;
  StepSched*             d_sched = nullptr;

  std::map<int, cudaGraphExec_t> graphs;

  // Host-buffer pipeline (nsm_compute_internal_force_host): K element chunks,
  // the copy of u in by node ranges ahead of them and the copy of f_int out
  // by node ranges behind them.  hp_e[j]..hp_e[j+1] are chunk j's elements;
  // nodes [0, hp_in[j+1]) cover every node of chunks 0..j; every element of
  // nodes [0, hp_ready[j+1]) is in chunks 0..j.
  int                      host_chunks = -1;  // requested (-1: by size)
  int                      hp_k = 0;          // chunks the cut tables were built for
  std::vector<int>         hp_e, hp_in, hp_ready;
  cudaStream_t             hp_stream[4] = {};  // copy in, elements (2), copy out
  std::vector<cudaEvent_t> hp_ev;              // [0]: start; then per chunk: in, elements, gathered
  double*                  d_stage_out = nullptr;

  // profiling
  bool                                              profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_elem, ev_node;
  size_t                                            ev_elem_used = 0, ev_node_used = 0;

  size_t elem_bytes() const { return precision == NSM_PRECISION_FP64 ? 8 : 4; }
};

namespace {

void free_all(nsm_model* m)
{
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);
  m->graphs.clear();
  void* ptrs[] = {m->d_conn, m->d_node_ptr, m->d_node_inc, m->d_node_slots, m->d_node_more, m->d_X,     m->d_u,         m->d_v,     m->d_a,
                  m->d_f,    m->d_fext,     m->d_mass,     m->d_inv_mass, m->d_geo,    m->d_ip,    m->d_Xf,
                  m->d_uf,   m->d_fe,   m->d_status,   m->d_step_base, m->d_scratch, m->d_stage,  m->d_out,   m->d_bc_slot,
                  m->d_bcs,  m->d_ibc_slot, m->d_ibcs,     m->d_sched, m->d_group_out, m->d_elem_group,
                  m->d_node_group, m->d_elem_off, m->d_mats, m->d_fallbacks, m->d_node_off, m->d_closure,
                  m->d_stage_out, m->d_expr_code, m->d_expr_start, m->d_bc_slot_node, m->d_bc_expr_val,
                  m->d_closure_geo, m->d_ip_n, m->d_state, m->d_state_n};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (cudaStream_t s : m->hp_stream)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : m->hp_ev) cudaEventDestroy(e);
  m->hp_ev.clear();
  for (auto& e : m->ev_elem) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  for (auto& e : m->ev_node) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  if (m->stream) cudaStreamDestroy(m->stream);
}

int read_status(nsm_model* m)
{
  int status = 0;
  NSM_CUDA(cudaMemcpyAsync(&status, m->d_status, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  NSM_CUDA(cudaMemsetAsync(m->d_status, 0, sizeof(int), m->stream));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  if (status & NSM_STATUS_BAD_JACOBIAN) return fail(NSM_ERR_BAD_JACOBIAN, "non-positive Jacobian (inverted element)");
  if (status & NSM_STATUS_NONFINITE) return fail(NSM_ERR_NONFINITE, "non-finite element force");
  if (status & NSM_STATUS_TIMEOUT) return fail(NSM_ERR_STATE, "a bounded tensor-core wait ran out (learned closure)");
  return NSM_OK;
}

// Per-node boundary-condition tables: the last line in deck order wins per
// (node, component), as each line overwrites the component it names.
int upload_bcs(nsm_model* m)
{
  if (!m->bcs_dirty) return NSM_OK;
  for (int pass = 0; pass < 2; pass++) {
    std::vector<int>    slot(m->N, -1);
    std::vector<NodeBC> table;
    std::vector<int>    slot_node;
    bool                any_expr = false;
    for (const BcLine& b : m->bcs) {
      bool initial = b.kind == NSM_BC_INITIAL_VELOCITY;
      if ((pass == 0) == initial) continue;  // pass 0: kinematic lines, pass 1: initial velocity
      for (int n : b.nodes) {
        if (slot[n] < 0) {
          slot[n] = (int)table.size();
          slot_node.push_back(n);
          NodeBC z;
          std::memset(&z, 0, sizeof(z));
          z.expr[0] = z.expr[1] = z.expr[2] = -1;
          table.push_back(z);
        }
        NodeBC& t          = table[slot[n]];
        t.kind[b.component]  = (int8_t)(initial ? 1 : (b.kind == NSM_BC_PRESCRIBED_VELOCITY ? 1 : 2));
        t.value[b.component] = b.value;
        t.expr[b.component]  = (int8_t)b.expr;
        any_expr             = any_expr || b.expr >= 0;
      }
    }
    int*&    d_slot = pass == 0 ? m->d_bc_slot : m->d_ibc_slot;
    NodeBC*& d_tab  = pass == 0 ? m->d_bcs : m->d_ibcs;
    if (d_tab) cudaFree(d_tab);
    d_tab = nullptr;
    if (!d_slot) NSM_CUDA(cudaMalloc(&d_slot, sizeof(int) * (size_t)(m->N > 0 ? m->N : 1)));
    if (!table.empty()) {
      NSM_CUDA(cudaMalloc(&d_tab, sizeof(NodeBC) * table.size()));
      NSM_CUDA(cudaMemcpyAsync(d_tab, table.data(), sizeof(NodeBC) * table.size(), cudaMemcpyHostToDevice,
                               m->stream));
    }
    if (m->N > 0)
      NSM_CUDA(cudaMemcpyAsync(d_slot, slot.data(), sizeof(int) * m->N, cudaMemcpyHostToDevice, m->stream));
    if (pass == 0) {  // kinematic conditions: the node of each slot, value space for expressions
      if (m->d_bc_slot_node) cudaFree(m->d_bc_slot_node);
      if (m->d_bc_expr_val) cudaFree(m->d_bc_expr_val);
      m->d_bc_slot_node = nullptr;
      m->d_bc_expr_val  = nullptr;
      m->num_bc_slots   = (int)table.size();
      m->bc_has_expr    = any_expr;
      if (any_expr) {
        NSM_CUDA(cudaMalloc(&m->d_bc_slot_node, sizeof(int) * slot_node.size()));
        NSM_CUDA(cudaMemcpyAsync(m->d_bc_slot_node, slot_node.data(), sizeof(int) * slot_node.size(),
                                 cudaMemcpyHostToDevice, m->stream));
        NSM_CUDA(cudaMalloc(&m->d_bc_expr_val, sizeof(double) * 6 * slot_node.size()));
        NSM_CUDA(cudaMemsetAsync(m->d_bc_expr_val, 0, sizeof(double) * 6 * slot_node.size(), m->stream));
      }
    }
    NSM_CUDA(cudaStreamSynchronize(m->stream));  // host vectors go out of scope
  }
  // expression programs
  if (m->d_expr_code) cudaFree(m->d_expr_code);
  if (m->d_expr_start) cudaFree(m->d_expr_start);
  m->d_expr_code  = nullptr;
  m->d_expr_start = nullptr;
  if (!m->expr_code.empty()) {
    NSM_CUDA(cudaMalloc(&m->d_expr_code, sizeof(nsm::ExprOp) * m->expr_code.size()));
    NSM_CUDA(cudaMalloc(&m->d_expr_start, sizeof(int) * m->expr_start.size()));
    NSM_CUDA(cudaMemcpy(m->d_expr_code, m->expr_code.data(), sizeof(nsm::ExprOp) * m->expr_code.size(),
                        cudaMemcpyHostToDevice));
    NSM_CUDA(cudaMemcpy(m->d_expr_start, m->expr_start.data(), sizeof(int) * m->expr_start.size(),
                        cudaMemcpyHostToDevice));
  }
  m->bcs_dirty = false;
  // captured graphs hold the old table's address
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);
  m->graphs.clear();
  return NSM_OK;
}

double* field_ptr(nsm_model* m, int field)
{
  switch (field) {
    case NSM_FIELD_REFERENCE_COORDINATE: return m->d_X;
    case NSM_FIELD_DISPLACEMENT: return m->d_u;
    case NSM_FIELD_VELOCITY: return m->d_v;
    case NSM_FIELD_ACCELERATION: return m->d_a;
    case NSM_FIELD_INTERNAL_FORCE: return m->d_f;
    case NSM_FIELD_EXTERNAL_FORCE: return m->d_fext;
    default: return nullptr;
  }
}

nsm::ElementArgs element_args(nsm_model* m, int k)
{
  nsm::ElementArgs a;
  a.E         = m->E;
  a.e_begin   = 0;
  a.ld_e      = m->ld_e;
  a.ld_n      = m->ld_n;
  a.conn      = m->d_conn;
  a.u         = m->d_u;
  a.uf        = m->d_uf;
  a.Xf        = m->d_Xf;
  a.geo       = m->d_geo;
  a.bulk      = m->K;
  a.shear     = m->G;
  a.model     = m->model;
  a.ip        = m->d_ip;
  a.fe        = m->d_fe;
  a.elem_group = m->d_elem_group;
  a.mats       = m->d_mats;
  a.num_groups = m->S;
  a.persistent = 0;
  a.store_ip  = (k < 0 || m->store_ip) ? 1 : 0;
  a.sched     = k < 0 ? nullptr : m->d_sched;
  a.step_base = m->d_step_base;
  a.k         = k;
  a.status    = m->d_status;
  return a;
}

nsm::BcExprTable expr_table(const nsm_model* m)
{
  return nsm::BcExprTable{m->d_expr_code, m->d_expr_start, m->d_X, m->ld_n};
}

nsm::NodeArgs node_args(nsm_model* m, int k_post, int k_pre, int gather_only)
{
  nsm::NodeArgs a;
  a.N           = m->N;
  a.n_begin     = 0;
  a.ld_n        = m->ld_n;
  a.ld_e        = m->ld_e;
  a.node_ptr    = m->d_node_ptr;
  a.node_inc    = m->d_node_inc;
  a.node_slots  = m->d_node_slots;
  a.node_more   = m->d_node_more;
  a.fe          = m->d_fe;
  a.fe_is_float = m->precision == NSM_PRECISION_FP64 ? 0 : 1;
  a.inv_mass    = m->d_inv_mass;
  a.bc_slot     = m->d_bc_slot;
  a.bcs         = m->d_bcs;
  a.sched       = m->d_sched;
  a.step_base   = m->d_step_base;
  a.node_group  = m->d_node_group;
  a.num_groups  = m->S;
  a.k_post      = k_post;
  a.k_pre       = k_pre;
  a.gather_only = gather_only;
  a.u           = m->d_u;
  a.v           = m->d_v;
  a.a           = m->d_a;
  a.f_int       = m->d_f;
  a.uf          = m->d_uf;
  a.closure       = m->d_closure;
  a.closure_first = m->closure_first;
  a.num_exact     = m->num_exact;
  a.node_off      = m->d_node_off;
  a.bc_expr_val   = m->bc_has_expr ? m->d_bc_expr_val : nullptr;
  a.num_bc_slots  = m->num_bc_slots;
  return a;
}

// The FP32 form reads an FP32 copy of u; refresh it after u is written from
// outside the node kernel.
cudaError_t sync_uf(nsm_model* m)
{
  if (!m->d_uf) return cudaSuccess;
  return nsm::launch_to_float(3 * m->ld_n, m->d_u, m->d_uf, m->stream);
}

bool has_callbacks(const nsm_model* m)
{
  for (const auto& c : m->block_cb)
    if (c.fn) return true;
  return false;
}

// The split step of a model with block-material callbacks: the buffers of
// steps n and n+1 alternate, the kinematics pass writes F (and the built-in
// blocks' sigma) at n+1, each callback writes its block's sigma and state,
// and the forces follow from the recorded sigma.
cudaError_t element_split(nsm_model* m, int k)
{
  std::swap(m->d_ip, m->d_ip_n);
  std::swap(m->d_state, m->d_state_n);
  double t_n = m->ci_t_prev, t_np1 = m->ci_t_cur;
  if (k >= 0) {
    const size_t s = (size_t)(m->steps_done + k);
    t_n            = m->h_time[s];
    t_np1          = m->h_time[s + 1];
  }
  const int        is_float = m->precision == NSM_PRECISION_FP64 ? 0 : 1;
  nsm::ElementArgs a        = element_args(m, k);
  cudaError_t      e        = nsm::launch_element_pass(a, is_float, 1, m->stream);
  for (size_t b = 0; b < m->block_cb.size() && e == cudaSuccess; b++) {
    const auto& cb = m->block_cb[b];
    if (!cb.fn || m->block_range[b].first < 0) continue;
    nsm_stress_request r;
    r.block        = (int)b;
    r.elem_begin   = m->block_range[b].first;
    r.elem_end     = m->block_range[b].second;
    r.precision    = m->precision;
    r.ld_e         = m->ld_e;
    r.records_n    = m->d_ip_n;
    r.records_np1  = m->d_ip;
    r.num_state    = m->num_state;
    r.state_n      = m->num_state > 0 ? m->d_state_n : nullptr;
    r.state_np1    = m->num_state > 0 ? m->d_state : nullptr;
    r.time_n       = t_n;
    r.time_np1     = t_np1;
    r.density      = m->h_mats[b].density;
    r.bulk_modulus = m->h_mats[b].bulk;
    r.shear_modulus = m->h_mats[b].shear;
    r.stream       = m->stream;
    if (cb.fn(cb.user, &r) != 0) {
      m->cb_failed = true;
      return cudaErrorLaunchFailure;  // reported as the callback's failure
    }
  }
  if (e == cudaSuccess) e = nsm::launch_element_pass(a, is_float, 2, m->stream);
  return e;
}

cudaError_t launch_element(nsm_model* m, int k)
{
  if (has_callbacks(m)) return element_split(m, k);
  nsm::ElementArgs a = element_args(m, k);
  if (m->closure) {
    nsm::mlp::MlpElementArgs ma;
    nsm::mlp::element_args(m->closure, &ma, nullptr, nullptr);
    ma.fallback_count = m->d_fallbacks;
    ma.geo            = m->d_closure_geo;
    return nsm::mlp::launch_element_mlp(a, ma, m->stream);
  }
  return m->precision == NSM_PRECISION_FP64 ? nsm::launch_element_fp64(a, m->elaunch, m->stream)
                                            : nsm::launch_element_fp32(a, m->elaunch, m->stream);
}

std::pair<cudaEvent_t, cudaEvent_t> next_events(std::vector<std::pair<cudaEvent_t, cudaEvent_t>>& pool, size_t& used)
{
  if (used == pool.size()) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    pool.push_back({a, b});
  }
  return pool[used++];
}

// One node launch of the time loop, after the values of its expression
// conditions when there are any.
cudaError_t node_step(nsm_model* m, int k_post, int k_pre)
{
  const nsm::NodeArgs a = node_args(m, k_post, k_pre, 0);
  if (m->bc_has_expr) {
    cudaError_t e = nsm::launch_bc_expr_values(a, m->d_bc_slot_node, expr_table(m), m->d_bc_expr_val, m->stream);
    if (e != cudaSuccess) return e;
  }
  return nsm::launch_node_update(a, m->stream);
}

// Launch sequence of a chunk of K schedule steps starting at the device base:
// node(pre 0); {element(k); node(post k, pre k+1)}; node(post K-1); base += K.
cudaError_t enqueue_chunk(nsm_model* m, int K, bool timed)
{
  cudaError_t e;
  if ((e = node_step(m, -1, 0)) != cudaSuccess) return e;
  for (int k = 0; k < K; k++) {
    if (timed) {
      auto ev = next_events(m->ev_elem, m->ev_elem_used);
      cudaEventRecord(ev.first, m->stream);
      if ((e = launch_element(m, k)) != cudaSuccess) return e;
      cudaEventRecord(ev.second, m->stream);
      auto en = next_events(m->ev_node, m->ev_node_used);
      cudaEventRecord(en.first, m->stream);
      if ((e = node_step(m, k, k + 1 < K ? k + 1 : -1)) != cudaSuccess) return e;
      cudaEventRecord(en.second, m->stream);
    } else {
      if ((e = launch_element(m, k)) != cudaSuccess) return e;
      if ((e = node_step(m, k, k + 1 < K ? k + 1 : -1)) != cudaSuccess) return e;
    }
  }
  return nsm::launch_advance_base(m->d_step_base, K, m->stream);
}

int get_graph(nsm_model* m, int K, cudaGraphExec_t* out)
{
  auto it = m->graphs.find(K);
  if (it != m->graphs.end()) {
    *out = it->second;
    return NSM_OK;
  }
  cudaGraph_t graph;
  NSM_CUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e  = enqueue_chunk(m, K, false);
  cudaError_t e2 = cudaStreamEndCapture(m->stream, &graph);
  if (e != cudaSuccess) return cuda_fail(e, "capture");
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  cudaGraphExec_t exec;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  m->graphs[K] = exec;
  *out         = exec;
  return NSM_OK;
}

}  // namespace

int nsm::set_last_error(int code, const char* msg) { return fail(code, msg); }
int nsm::model_num_nodes(const nsm_model* m) { return m->N; }

extern "C" {

const char* nsm_last_error(void) { return g_error.c_str(); }
int         nsm_abi_version(void) { return NSM_ABI_VERSION; }

}  // extern "C"

namespace {

// One handle over S samples: the samples' meshes are concatenated (node and
// element ids offset per sample) and each node carries its sample's time
// schedule.  Materials: `num_mats` entries, element e uses
// materials[elem_mat[e]] (global element ids); elem_mat null means material
// g for the elements of sample g when num_mats == S (ensembles), or material
// 0 (one material).  A single mesh is S = 1.
int create_impl(int S, const nsm_mesh_desc* meshes, int num_mats, const nsm_material* materials,
                const int* elem_mat, const nsm_options* options, nsm_model** out)
{
  if (!meshes || !materials || !out || S < 1 || num_mats < 1) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  if (!elem_mat && num_mats != 1 && num_mats != S) return fail(NSM_ERR_INVALID_ARGUMENT, "materials per element needed");
  *out = nullptr;
  for (int b = 0; b < num_mats; b++) {
    const nsm_material& mat = materials[b];
    if (mat.model != NSM_MATERIAL_NEOHOOKEAN && mat.model != NSM_MATERIAL_ELASTIC)
      return fail(NSM_ERR_INVALID_ARGUMENT, "unknown material model");
    if (!(mat.density > 0) || !(mat.bulk_modulus > 0) || !(mat.shear_modulus >= 0))
      return fail(NSM_ERR_INVALID_ARGUMENT, "invalid material parameters");
  }
  std::vector<int> node_off(S + 1, 0), elem_off(S + 1, 0);
  for (int g = 0; g < S; g++) {
    const nsm_mesh_desc& mesh = meshes[g];
    if (mesh.num_nodes < 0 || mesh.num_elem < 0 || (mesh.num_elem > 0 && (!mesh.coords || !mesh.conn)))
      return fail(NSM_ERR_INVALID_ARGUMENT, "invalid mesh");
    for (long i = 0; i < 8L * mesh.num_elem; i++)
      if (mesh.conn[i] < 0 || mesh.conn[i] >= mesh.num_nodes)
        return fail(NSM_ERR_INVALID_ARGUMENT, "connectivity out of range");
    if ((long)node_off[g] + mesh.num_nodes > 2000000000L || (long)elem_off[g] + mesh.num_elem > 250000000L)
      return fail(NSM_ERR_INVALID_ARGUMENT, "ensemble too large for 32-bit ids");
    node_off[g + 1] = node_off[g] + mesh.num_nodes;
    elem_off[g + 1] = elem_off[g] + mesh.num_elem;
  }
  const int N = node_off[S], E = elem_off[S];
  if (elem_mat) {
    // materials of a multi-block mesh: blocks are contiguous in element order,
    // which is the reference's block-by-block assembly order
    for (int e = 0; e < E; e++) {
      if (elem_mat[e] < 0 || elem_mat[e] >= num_mats) return fail(NSM_ERR_INVALID_ARGUMENT, "block index out of range");
      if (e > 0 && elem_mat[e] < elem_mat[e - 1])
        return fail(NSM_ERR_INVALID_ARGUMENT, "elements must be ordered by block");
    }
  }

  nsm_model* m = new nsm_model();
  m->N = N;
  m->E = E;
  m->S = S;
  m->node_off = node_off;
  m->elem_off = elem_off;
  m->ld_n = pad(N > 0 ? N : 1, 64);
  m->ld_e = pad(E > 0 ? E : 1, 64);
  if (options) {
    m->precision   = options->precision;
    m->store_ip    = options->store_ip_data;
    m->device      = options->device;
    m->graph_steps = options->graph_steps > 0 ? options->graph_steps : 50;
  }
  if (m->precision != NSM_PRECISION_FP64 && m->precision != NSM_PRECISION_FP32_MIXED) {
    delete m;
    return fail(NSM_ERR_INVALID_ARGUMENT, "unknown precision");
  }
  // default launch shapes, the fastest measured at 128^3: FP64 one thread per
  // element; FP32 the persistent grid with the nodal values staged ahead
  // the measured fastest shapes at 128^3: FP64 registers bounded for 3 CTAs of
  // 128 per SM (5.34 ms against 5.38 unbounded), FP32 the staged persistent grid
  m->elaunch = m->precision == NSM_PRECISION_FP64 ? nsm::ElementLaunch{128, 0, 3, 0} : nsm::ElementLaunch{128, 1, 3, 1};
  m->density   = materials[0].density;
  m->K         = materials[0].bulk_modulus;
  m->G         = materials[0].shear_modulus;
  m->model     = materials[0].model;
  m->num_mats  = num_mats;
  std::vector<nsm::GroupMaterial> gm(num_mats);
  for (int b = 0; b < num_mats; b++)
    gm[b] = nsm::GroupMaterial{materials[b].bulk_modulus, materials[b].shear_modulus, materials[b].density,
                               std::sqrt(materials[b].bulk_modulus / materials[b].density), materials[b].model, 0};
  m->h_mats = gm;
  m->block_cb.assign(num_mats, nsm_model::BlockCallback{});
  m->block_range.assign(num_mats, std::make_pair(-1, -1));

  auto bail = [&](int code) {
    free_all(m);
    delete m;
    return code;
  };
#define NSM_CUDA_B(call)                                       \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) return bail(cuda_fail(_e, #call));  \
  } while (0)

  NSM_CUDA_B(cudaSetDevice(m->device));
  NSM_CUDA_B(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  const size_t nb = sizeof(double) * 3 * m->ld_n, eb = m->elem_bytes();
  NSM_CUDA_B(cudaMalloc(&m->d_conn, sizeof(int) * 8 * m->ld_e));
  NSM_CUDA_B(cudaMalloc(&m->d_node_ptr, sizeof(int) * (N + 1)));
  NSM_CUDA_B(cudaMalloc(&m->d_node_inc, sizeof(int) * (8L * E > 0 ? 8L * E : 1)));
  NSM_CUDA_B(cudaMalloc(&m->d_node_slots, sizeof(int) * (m->ld_n > 0 ? 8 * m->ld_n : 1)));
  NSM_CUDA_B(cudaMalloc(&m->d_node_more, sizeof(unsigned) * (m->ld_n > 0 ? (m->ld_n + 31) / 32 : 1)));
  double** nodal[] = {&m->d_X, &m->d_u, &m->d_v, &m->d_a, &m->d_f, &m->d_fext};
  for (double** p : nodal) {
    NSM_CUDA_B(cudaMalloc(p, nb));
    NSM_CUDA_B(cudaMemsetAsync(*p, 0, nb, m->stream));
  }
  NSM_CUDA_B(cudaMalloc(&m->d_mass, sizeof(double) * m->ld_n));
  NSM_CUDA_B(cudaMalloc(&m->d_inv_mass, sizeof(double) * m->ld_n));
  NSM_CUDA_B(cudaMalloc(&m->d_geo, sizeof(double) * 8 * nsm::kGeoPerPoint * m->ld_e));
  NSM_CUDA_B(cudaMalloc(&m->d_ip, eb * nsm::kIpRecord * 8 * m->ld_e));
  NSM_CUDA_B(cudaMalloc(&m->d_fe, eb * 24 * m->ld_e));
  NSM_CUDA_B(cudaMemsetAsync(m->d_ip, 0, eb * nsm::kIpRecord * 8 * m->ld_e, m->stream));
  NSM_CUDA_B(nsm::launch_ip_identity(E, m->ld_e, m->d_ip, m->precision == NSM_PRECISION_FP64 ? 0 : 1, m->stream));
  NSM_CUDA_B(cudaMemsetAsync(m->d_fe, 0, eb * 24 * m->ld_e, m->stream));
  if (m->precision == NSM_PRECISION_FP32_MIXED) {
    NSM_CUDA_B(cudaMalloc(&m->d_Xf, sizeof(float) * 3 * m->ld_n));
    NSM_CUDA_B(cudaMalloc(&m->d_uf, sizeof(float) * 3 * m->ld_n));
    NSM_CUDA_B(cudaMemsetAsync(m->d_uf, 0, sizeof(float) * 3 * m->ld_n, m->stream));
  }
  NSM_CUDA_B(cudaMalloc(&m->d_status, sizeof(int)));
  NSM_CUDA_B(cudaMemsetAsync(m->d_status, 0, sizeof(int), m->stream));
  NSM_CUDA_B(cudaMalloc(&m->d_step_base, sizeof(int)));
  NSM_CUDA_B(cudaMemsetAsync(m->d_step_base, 0, sizeof(int), m->stream));
  NSM_CUDA_B(cudaMalloc(&m->d_out, sizeof(double) * 8));
  NSM_CUDA_B(cudaMalloc(&m->d_group_out, sizeof(double) * S));
  NSM_CUDA_B(cudaMalloc(&m->d_stage, nb));
  NSM_CUDA_B(cudaMalloc(&m->d_mats, sizeof(nsm::GroupMaterial) * num_mats));
  NSM_CUDA_B(cudaMemcpyAsync(m->d_mats, gm.data(), sizeof(nsm::GroupMaterial) * num_mats, cudaMemcpyHostToDevice,
                             m->stream));
  NSM_CUDA_B(cudaMalloc(&m->d_elem_off, sizeof(int) * (S + 1)));
  NSM_CUDA_B(cudaMemcpyAsync(m->d_elem_off, elem_off.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, m->stream));
  size_t scratch = sizeof(double) * (E > 0 ? (size_t)E : 1);
  if (scratch < sizeof(double) * 2 * nsm::kEnergyBlocks) scratch = sizeof(double) * 2 * nsm::kEnergyBlocks;
  NSM_CUDA_B(cudaMalloc(&m->d_scratch, scratch + sizeof(double) * 1024));

  // host layouts -> device planes
  {
    std::vector<int>    conn_soa((size_t)8 * m->ld_e, 0);
    std::vector<double> X((size_t)3 * m->ld_n, 0.0);
    std::vector<int>    egroup, ngroup;
    if (num_mats > 1) egroup.resize(E);
    if (S > 1) ngroup.resize(N);
    std::vector<int> gconn((size_t)8 * E);
    for (int g = 0; g < S; g++) {
      const nsm_mesh_desc& mesh = meshes[g];
      for (long e = 0; e < mesh.num_elem; e++) {
        long ge = elem_off[g] + e;
        for (int c = 0; c < 8; c++) {
          int gid                          = node_off[g] + mesh.conn[8 * e + c];
          conn_soa[(size_t)c * m->ld_e + ge] = gid;
          gconn[8 * ge + c]                = gid;
        }
        if (num_mats > 1) egroup[ge] = elem_mat ? elem_mat[ge] : g;
        const int b = num_mats > 1 ? egroup[ge] : 0;  // blocks are contiguous (checked above)
        if (m->block_range[b].first < 0) m->block_range[b].first = (int)ge;
        m->block_range[b].second = (int)ge + 1;
      }
      for (long n = 0; n < mesh.num_nodes; n++) {
        long gn = node_off[g] + n;
        for (int k = 0; k < 3; k++) X[(size_t)k * m->ld_n + gn] = mesh.coords[3 * n + k];
        if (S > 1) ngroup[gn] = g;
      }
    }
    // node -> (element, corner) incidence in increasing element order
    std::vector<int> ptr(N + 1, 0), inc((size_t)8 * E);
    for (long i = 0; i < 8L * E; i++) ptr[gconn[i] + 1]++;
    for (int n = 0; n < N; n++) ptr[n + 1] += ptr[n];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (long i = 0; i < 8L * E; i++) inc[fill[gconn[i]]++] = (int)i;
    // the same incidences, the first 8 of each node slot-major, so that the
    // node kernel loads them without reading the node's CSR range first
    std::vector<int>      slots((size_t)8 * m->ld_n, -1);
    std::vector<unsigned> more((m->ld_n + 31) / 32, 0u);
    for (int n = 0; n < N; n++) {
      for (int j = 0; j < 8 && ptr[n] + j < ptr[n + 1]; j++) slots[(size_t)j * m->ld_n + n] = inc[ptr[n] + j];
      if (ptr[n + 1] - ptr[n] > 8) more[n >> 5] |= 1u << (n & 31);
    }
    if (m->ld_n > 0) {
      NSM_CUDA_B(cudaMemcpyAsync(m->d_node_slots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice,
                                 m->stream));
      NSM_CUDA_B(cudaMemcpyAsync(m->d_node_more, more.data(), sizeof(unsigned) * more.size(),
                                 cudaMemcpyHostToDevice, m->stream));
    }
    NSM_CUDA_B(cudaMemcpyAsync(m->d_conn, conn_soa.data(), sizeof(int) * conn_soa.size(), cudaMemcpyHostToDevice,
                               m->stream));
    NSM_CUDA_B(cudaMemcpyAsync(m->d_X, X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice, m->stream));
    if (m->d_Xf) NSM_CUDA_B(nsm::launch_to_float(3 * m->ld_n, m->d_X, m->d_Xf, m->stream));
    NSM_CUDA_B(cudaMemcpyAsync(m->d_node_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice,
                               m->stream));
    if (E > 0)
      NSM_CUDA_B(cudaMemcpyAsync(m->d_node_inc, inc.data(), sizeof(int) * inc.size(), cudaMemcpyHostToDevice,
                                 m->stream));
    if (num_mats > 1) {
      NSM_CUDA_B(cudaMalloc(&m->d_elem_group, sizeof(int) * (E > 0 ? E : 1)));
      if (E > 0)
        NSM_CUDA_B(cudaMemcpyAsync(m->d_elem_group, egroup.data(), sizeof(int) * E, cudaMemcpyHostToDevice, m->stream));
    }
    if (S > 1) {
      NSM_CUDA_B(cudaMalloc(&m->d_node_group, sizeof(int) * (N > 0 ? N : 1)));
      if (N > 0)
        NSM_CUDA_B(cudaMemcpyAsync(m->d_node_group, ngroup.data(), sizeof(int) * N, cudaMemcpyHostToDevice, m->stream));
    }
    NSM_CUDA_B(nsm::upload_shape_tables(m->stream));

    // setup: geometry, lumped mass, critical time step per sample
    double* me = nullptr;
    NSM_CUDA_B(cudaMalloc(&me, sizeof(double) * 8 * m->ld_e));
    nsm::SetupArgs s;
    s.N          = N;
    s.E          = E;
    s.num_groups = S;
    s.elem_group = m->d_elem_group;
    s.elem_off   = m->d_elem_off;
    s.mats       = m->d_mats;
    s.ld_n       = m->ld_n;
    s.ld_e       = m->ld_e;
    s.conn       = m->d_conn;
    s.X          = m->d_X;
    s.node_ptr   = m->d_node_ptr;
    s.node_inc   = m->d_node_inc;
    s.geo        = m->d_geo;
    s.me         = me;
    s.dt_elem    = m->d_scratch;
    s.dt_partial = m->d_scratch + (scratch / sizeof(double));
    s.dt_out     = m->d_group_out;
    s.mass       = m->d_mass;
    s.inv_mass   = m->d_inv_mass;
    s.status     = m->d_status;
    cudaError_t e = nsm::launch_setup(s, m->stream);  // also for no elements: mass 0, the largest step
    m->dt_group.assign(S, 1.7976931348623157e308);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(m->dt_group.data(), m->d_group_out, sizeof(double) * S, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);  // host vectors live until here
    cudaFree(me);
    if (e != cudaSuccess) return bail(cuda_fail(e, "setup"));
    m->dt_crit = 1.7976931348623157e308;
    for (double d : m->dt_group)
      if (d < m->dt_crit) m->dt_crit = d;
  }
  int st = read_status(m);
  if (st != NSM_OK) return bail(st);
  int bc = upload_bcs(m);
  if (bc != NSM_OK) return bail(bc);
#undef NSM_CUDA_B
  *out = m;
  return NSM_OK;
}

}  // namespace

extern "C" {

static nsm_material as_material(const nsm_neohookean& m)
{
  return nsm_material{NSM_MATERIAL_NEOHOOKEAN, 0, m.density, m.bulk_modulus, m.shear_modulus};
}

int nsm_create(const nsm_mesh_desc* mesh, const nsm_neohookean* material, const nsm_options* options,
               nsm_model** out)
{
  if (!material) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  const nsm_material mat = as_material(*material);
  return create_impl(1, mesh, 1, &mat, nullptr, options, out);
}

int nsm_create_ensemble(int num_samples, const nsm_mesh_desc* meshes, const nsm_neohookean* materials,
                        const nsm_options* options, nsm_model** out)
{
  if (!materials || num_samples < 1) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<nsm_material> mats(num_samples);
  for (int g = 0; g < num_samples; g++) mats[g] = as_material(materials[g]);
  return create_impl(num_samples, meshes, num_samples, mats.data(), nullptr, options, out);
}

int nsm_create_blocks(const nsm_mesh_desc* mesh, int num_blocks, const int* elem_block, const nsm_material* materials,
                      const nsm_options* options, nsm_model** out)
{
  if (!mesh || num_blocks < 1 || (num_blocks > 1 && !elem_block)) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  return create_impl(1, mesh, num_blocks, materials, num_blocks > 1 ? elem_block : nullptr, options, out);
}

int nsm_create_uq(const nsm_mesh_desc* mesh, int num_blocks, const int* elem_block, const nsm_material* nominal,
                  int num_exact, const double* exact_bulk, const double* exact_shear, int num_approx,
                  const double* coefficients, const nsm_options* options, nsm_model** out)
{
  if (!mesh || !nominal || !out || num_blocks < 1 || num_exact < 0 || num_approx < 0 ||
      (num_blocks > 1 && !elem_block) || (num_exact > 0 && (!exact_bulk || !exact_shear)) ||
      (num_approx > 0 && !coefficients))
    return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  const int S = 1 + num_exact + num_approx, B = num_blocks, full = 1 + num_exact;
  // trajectories: the nominal, the exact samples (elements, own moduli), the
  // approximate samples (nodes only, force from the closure)
  std::vector<nsm_mesh_desc> meshes(S, *mesh);
  for (int s = full; s < S; s++) meshes[s] = nsm_mesh_desc{mesh->num_nodes, 0, mesh->coords, nullptr};
  std::vector<nsm_material> mats((size_t)full * B);
  for (int k = 0; k < full; k++)
    for (int b = 0; b < B; b++) {
      nsm_material mt = nominal[b];
      if (k > 0) {
        mt.bulk_modulus  = exact_bulk[(size_t)(k - 1) * B + b];
        mt.shear_modulus = exact_shear[(size_t)(k - 1) * B + b];
      }
      mats[(size_t)k * B + b] = mt;
    }
  std::vector<int> emat((size_t)full * mesh->num_elem);
  for (int k = 0; k < full; k++)
    for (int e = 0; e < mesh->num_elem; e++)
      emat[(size_t)k * mesh->num_elem + e] = k * B + (B > 1 ? elem_block[e] : 0);
  int rc = create_impl(S, meshes.data(), full * B, mats.data(), emat.data(), options, out);
  if (rc != NSM_OK) return rc;
  nsm_model* m = *out;
  cudaError_t e = cudaSuccess;
  if (num_approx > 0) {
    // the approximate samples use the nominal's lumped mass (mass[i / 3],
    // src/uq/nimble_uq_model_data.cc:218-234)
    const size_t nb = sizeof(double) * mesh->num_nodes;
    for (int s = full; s < S && e == cudaSuccess; s++) {
      e = cudaMemcpyAsync(m->d_mass + m->node_off[s], m->d_mass, nb, cudaMemcpyDeviceToDevice, m->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(m->d_inv_mass + m->node_off[s], m->d_inv_mass, nb, cudaMemcpyDeviceToDevice, m->stream);
    }
    if (e == cudaSuccess) e = cudaMalloc(&m->d_closure, sizeof(double) * num_approx * (num_exact + 1));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(m->d_closure, coefficients, sizeof(double) * num_approx * (num_exact + 1),
                          cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_node_off, sizeof(int) * (S + 1));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(m->d_node_off, m->node_off.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    m->closure_first = full;
    m->num_exact     = num_exact;
  }
  if (e != cudaSuccess) {
    nsm_destroy(m);
    *out = nullptr;
    return cuda_fail(e, "nsm_create_uq");
  }
  return NSM_OK;
}

int nsm_ensemble_offsets(nsm_model* m, int* node_offsets, int* elem_offsets)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  for (int g = 0; g <= m->S; g++) {
    if (node_offsets) node_offsets[g] = m->node_off[g];
    if (elem_offsets) elem_offsets[g] = m->elem_off[g];
  }
  return NSM_OK;
}

int nsm_ensemble_time_steps(nsm_model* m, double* dt)
{
  if (!m || !dt) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  for (int g = 0; g < m->S; g++) dt[g] = m->dt_group[g];
  return NSM_OK;
}

int nsm_ensemble_max_abs(nsm_model* m, int field, int component, const int* nodes, int count, double* out)
{
  if (!m || !out || (count > 0 && !nodes)) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  double* src = field_ptr(m, field);
  if (!src || component < 0 || component > 2) return fail(NSM_ERR_INVALID_ARGUMENT, "unknown field");
  for (int i = 0; i < count; i++)
    if (nodes[i] < 0 || nodes[i] >= m->N) return fail(NSM_ERR_INVALID_ARGUMENT, "node id out of range");
  NSM_CUDA(cudaSetDevice(m->device));
  int* d_nodes = nullptr;
  if (count > 0) {
    NSM_CUDA(cudaMalloc(&d_nodes, sizeof(int) * count));
    NSM_CUDA(cudaMemcpyAsync(d_nodes, nodes, sizeof(int) * count, cudaMemcpyHostToDevice, m->stream));
  }
  cudaError_t e = nsm::launch_group_max_abs(count, d_nodes, src, m->ld_n, component, m->d_node_group, m->S,
                                            m->d_group_out, m->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, m->d_group_out, sizeof(double) * m->S, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (d_nodes) cudaFree(d_nodes);
  if (e != cudaSuccess) return cuda_fail(e, "nsm_ensemble_max_abs");
  return NSM_OK;
}

int nsm_destroy(nsm_model* m)
{
  if (!m) return NSM_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  free_all(m);
  delete m;
  return NSM_OK;
}

int nsm_add_boundary_condition(nsm_model* m, int kind, int component, double value, const int* nodes, int count)
{
  if (!m || (count > 0 && !nodes)) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  if (kind < NSM_BC_INITIAL_VELOCITY || kind > NSM_BC_PRESCRIBED_DISPLACEMENT)
    return fail(NSM_ERR_INVALID_ARGUMENT, "unknown boundary condition kind");
  if (component < 0 || component > 2) return fail(NSM_ERR_INVALID_ARGUMENT, "unknown coordinate");
  BcLine b{kind, component, value, std::vector<int>(nodes, nodes + count)};
  for (int n : b.nodes)
    if (n < 0 || n >= m->N) return fail(NSM_ERR_INVALID_ARGUMENT, "node set entry out of range");
  m->bcs.push_back(std::move(b));
  m->bcs_dirty = true;  // uploaded when next needed
  return NSM_OK;
}

int nsm_add_boundary_condition_expression(nsm_model* m, int kind, int component, const char* expression,
                                          const int* nodes, int count)
{
  if (!m || !expression || (count > 0 && !nodes)) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  if (kind < NSM_BC_INITIAL_VELOCITY || kind > NSM_BC_PRESCRIBED_DISPLACEMENT)
    return fail(NSM_ERR_INVALID_ARGUMENT, "unknown boundary condition kind");
  if (component < 0 || component > 2) return fail(NSM_ERR_INVALID_ARGUMENT, "unknown coordinate");
  if ((int)m->expr_start.size() - 1 >= 127) return fail(NSM_ERR_INVALID_ARGUMENT, "more than 127 expressions");
  for (int i = 0; i < count; i++)
    if (nodes[i] < 0 || nodes[i] >= m->N) return fail(NSM_ERR_INVALID_ARGUMENT, "node set entry out of range");
  const std::string err = nsm::compile_bc_expression(expression, m->expr_code);
  if (!err.empty()) return fail(NSM_ERR_INVALID_ARGUMENT, ("boundary condition expression: " + err).c_str());
  m->expr_start.push_back((int)m->expr_code.size());
  BcLine b{kind, component, 0.0, std::vector<int>(nodes, nodes + count), (int)m->expr_start.size() - 2};
  m->bcs.push_back(std::move(b));
  m->bcs_dirty = true;
  return NSM_OK;
}

int nsm_bc_expression_eval(const char* expression, double x, double y, double z, double t, double* value)
{
  if (!expression || !value) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<nsm::ExprOp> code;
  const std::string        err = nsm::compile_bc_expression(expression, code);
  if (!err.empty()) return fail(NSM_ERR_INVALID_ARGUMENT, ("boundary condition expression: " + err).c_str());
  *value = nsm::eval_bc_expression_host(code.data(), (int)code.size(), x, y, z, t);
  return NSM_OK;
}

int nsm_compute_lumped_mass(nsm_model* m, double* mass)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  if (mass && m->N > 0) {
    NSM_CUDA(cudaMemcpyAsync(mass, m->d_mass, sizeof(double) * m->N, cudaMemcpyDeviceToHost, m->stream));
    NSM_CUDA(cudaStreamSynchronize(m->stream));
  }
  return NSM_OK;
}

int nsm_critical_time_step(nsm_model* m, double* dt)
{
  if (!m || !dt) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  *dt = m->dt_crit;
  return NSM_OK;
}

int nsm_apply_initial_conditions(nsm_model* m)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  int r = upload_bcs(m);
  if (r) return r;
  if (m->d_ibcs)
    NSM_CUDA(nsm::launch_apply_bc(m->N, m->ld_n, m->d_ibc_slot, m->d_ibcs, 0.0, 0.0, expr_table(m), m->d_u, m->d_v,
                                  m->stream));
  return NSM_OK;
}

int nsm_apply_kinematic_conditions(nsm_model* m, double t_cur, double t_prev)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  int r = upload_bcs(m);
  if (r) return r;
  if (m->d_bcs)
    NSM_CUDA(nsm::launch_apply_bc(m->N, m->ld_n, m->d_bc_slot, m->d_bcs, t_cur - t_prev, t_cur, expr_table(m), m->d_u,
                                  m->d_v, m->stream));
  return NSM_OK;
}

int nsm_set_node_field(nsm_model* m, int field, const double* values)
{
  if (!m || !values) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  double* dst = field_ptr(m, field);
  if (!dst) return fail(NSM_ERR_INVALID_ARGUMENT, "unknown field");
  if (field == NSM_FIELD_REFERENCE_COORDINATE) return fail(NSM_ERR_INVALID_ARGUMENT, "reference coordinates are fixed");
  if (field == NSM_FIELD_EXTERNAL_FORCE)  // ModelData::ComputeExternalForce zeroes it every step
    return fail(NSM_ERR_INVALID_ARGUMENT, "the external force is zero on this path");
  NSM_CUDA(cudaSetDevice(m->device));
  if (m->N == 0) return NSM_OK;
  NSM_CUDA(cudaMemcpyAsync(m->d_stage, values, sizeof(double) * 3 * m->N, cudaMemcpyHostToDevice, m->stream));
  NSM_CUDA(nsm::launch_node_aos_to_soa(m->N, m->ld_n, m->d_stage, dst, nullptr, m->stream));
  if (dst == m->d_u) NSM_CUDA(sync_uf(m));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  return NSM_OK;
}

int nsm_get_node_field(nsm_model* m, int field, double* values)
{
  if (!m || !values) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  double* src = field_ptr(m, field);
  if (!src) return fail(NSM_ERR_INVALID_ARGUMENT, "unknown field");
  NSM_CUDA(cudaSetDevice(m->device));
  if (m->N == 0) return NSM_OK;
  NSM_CUDA(nsm::launch_node_soa_to_aos(m->N, m->ld_n, src, m->d_stage, m->stream));
  NSM_CUDA(cudaMemcpyAsync(values, m->d_stage, sizeof(double) * 3 * m->N, cudaMemcpyDeviceToHost, m->stream));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  return NSM_OK;
}

int nsm_compute_internal_force(nsm_model* m, double time_previous, double time_current, int)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  m->ci_t_prev  = time_previous;  // the step's times for block-material callbacks
  m->ci_t_cur   = time_current;
  m->cb_failed  = false;
  cudaError_t e = launch_element(m, -1);
  if (m->cb_failed) return fail(NSM_ERR_STATE, "a block-material callback failed");
  NSM_CUDA(e);
  NSM_CUDA(nsm::launch_node_update(node_args(m, -1, -1, 1), m->stream));
  return read_status(m);
}

namespace {

// Chunks of the host-buffer pipeline: none for the closures (the learned
// closure's kernel runs over all elements; a UQ sample's nodes gather the
// forces of other samples' elements) or a small mesh.
int host_chunk_count(const nsm_model* m)
{
  if (m->closure || m->d_closure || has_callbacks(m)) return 1;
  // default: measured fastest at 128^3 (FP64 8 chunks, 5.64 ms; FP32 4 chunks,
  // 0.63 ms, where each chunk's launches weigh more against 0.37 ms of device work)
  const int k_default = m->precision == NSM_PRECISION_FP64 ? 8 : 4;
  int       k         = m->host_chunks > 0 ? m->host_chunks : (m->E >= (1 << 18) ? k_default : 1);
  if (k > m->E) k = m->E > 0 ? m->E : 1;
  return k;
}

// Cut tables for K chunks from the connectivity (copied back once per K).
cudaError_t build_host_pipe(nsm_model* m, int K)
{
  const int        E = m->E, N = m->N;
  std::vector<int> conn((size_t)8 * m->ld_e);
  cudaError_t      err = cudaMemcpy(conn.data(), m->d_conn, sizeof(int) * conn.size(), cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) return err;
  std::vector<int> elem_hi(E);      // largest node of elements 0..e
  std::vector<int> node_last(N, -1);  // largest element of node n, then of nodes 0..n
  int              hi = -1;
  for (int e = 0; e < E; e++) {
    for (int c = 0; c < 8; c++) {
      const int id = conn[(size_t)c * m->ld_e + e];
      hi           = id > hi ? id : hi;
      if (e > node_last[id]) node_last[id] = e;
    }
    elem_hi[e] = hi;
  }
  for (int n = 1; n < N; n++) node_last[n] = node_last[n] > node_last[n - 1] ? node_last[n] : node_last[n - 1];
  m->hp_e.assign(K + 1, 0);
  m->hp_in.assign(K + 1, 0);
  m->hp_ready.assign(K + 1, 0);
  for (int j = 1; j <= K; j++) {
    m->hp_e[j]     = (int)((long)E * j / K);
    const int need = m->hp_e[j] > 0 ? elem_hi[m->hp_e[j] - 1] + 1 : 0;
    m->hp_in[j]    = j == K ? N : (need > m->hp_in[j - 1] ? need : m->hp_in[j - 1]);
    // first node with an element at or after the chunk's end
    const int* r   = std::lower_bound(node_last.data(), node_last.data() + N, m->hp_e[j]);
    m->hp_ready[j] = j == K ? N : (int)(r - node_last.data());
  }
  if ((int)m->hp_ev.size() < 1 + 3 * K) {
    for (cudaEvent_t e : m->hp_ev) cudaEventDestroy(e);
    m->hp_ev.assign(1 + 3 * K, nullptr);
    for (auto& e : m->hp_ev)
      if ((err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming)) != cudaSuccess) return err;
  }
  for (auto& s : m->hp_stream)
    if (!s && (err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return err;
  if (!m->d_stage_out && (err = cudaMalloc(&m->d_stage_out, sizeof(double) * 3 * (size_t)N)) != cudaSuccess)
    return err;
  m->hp_k = K;
  return cudaSuccess;
}

// The pipelined host-buffer evaluation: every element's arithmetic and every
// node's gather order are those of the one-launch path, so the result is
// bitwise the same.
cudaError_t internal_force_pipelined(nsm_model* m, const double* u_host, double* f_host, int K)
{
  cudaStream_t s_in = m->hp_stream[0], s_out = m->hp_stream[3];
  cudaStream_t s_el[2] = {m->hp_stream[1], m->hp_stream[2]};
  cudaEvent_t* ev      = m->hp_ev.data();  // ev[0] start; ev[1 + 3j + {0, 1, 2}] in, elements, gathered
  cudaError_t  err     = cudaEventRecord(ev[0], m->stream);  // earlier work on the state is done first
  if (err == cudaSuccess) err = cudaStreamWaitEvent(s_in, ev[0], 0);
  for (int j = 0; j < K && err == cudaSuccess; j++) {
    const int n0 = m->hp_in[j], n1 = m->hp_in[j + 1];
    if (n1 > n0) {
      err = cudaMemcpyAsync(m->d_stage + 3L * n0, u_host + 3L * n0, sizeof(double) * 3 * (size_t)(n1 - n0),
                            cudaMemcpyHostToDevice, s_in);
      if (err == cudaSuccess)
        err = nsm::launch_node_aos_to_soa(n1 - n0, m->ld_n, m->d_stage + 3L * n0, m->d_u + n0,
                                          m->d_uf ? m->d_uf + n0 : nullptr, s_in);
    }
    if (err == cudaSuccess) err = cudaEventRecord(ev[1 + 3 * j], s_in);
  }
  for (int j = 0; j < K && err == cudaSuccess; j++) {
    cudaStream_t s = s_el[j & 1];
    err            = cudaStreamWaitEvent(s, ev[1 + 3 * j], 0);
    if (err == cudaSuccess) {
      nsm::ElementArgs a = element_args(m, -1);
      a.e_begin          = m->hp_e[j];
      a.E                = m->hp_e[j + 1];
      err = m->precision == NSM_PRECISION_FP64 ? nsm::launch_element_fp64(a, m->elaunch, s)
                                               : nsm::launch_element_fp32(a, m->elaunch, s);
    }
    if (err == cudaSuccess) err = cudaEventRecord(ev[2 + 3 * j], s);
  }
  for (int j = 0; j < K && err == cudaSuccess; j++) {
    // chunks 0..j done: the last one on each element stream
    err = cudaStreamWaitEvent(m->stream, ev[2 + 3 * j], 0);
    if (err == cudaSuccess && j > 0) err = cudaStreamWaitEvent(m->stream, ev[2 + 3 * (j - 1)], 0);
    const int r0 = m->hp_ready[j], r1 = m->hp_ready[j + 1];
    if (err == cudaSuccess && r1 > r0) {
      nsm::NodeArgs a = node_args(m, -1, -1, 1);
      a.n_begin       = r0;
      a.N             = r1;
      err             = nsm::launch_node_update(a, m->stream);
      if (err == cudaSuccess)
        err = nsm::launch_node_soa_to_aos(r1 - r0, m->ld_n, m->d_f + r0, m->d_stage_out + 3L * r0, m->stream);
    }
    if (err == cudaSuccess) err = cudaEventRecord(ev[3 + 3 * j], m->stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(s_out, ev[3 + 3 * j], 0);
    if (err == cudaSuccess && r1 > r0)
      err = cudaMemcpyAsync(f_host + 3L * r0, m->d_stage_out + 3L * r0, sizeof(double) * 3 * (size_t)(r1 - r0),
                            cudaMemcpyDeviceToHost, s_out);
  }
  if (err == cudaSuccess) err = cudaStreamSynchronize(s_out);
  return err;
}

}  // namespace

int nsm_set_host_chunks(nsm_model* m, int chunks)
{
  if (!m || chunks < 0 || chunks > 256) return fail(NSM_ERR_INVALID_ARGUMENT, "invalid chunk count");
  m->host_chunks = chunks == 0 ? -1 : chunks;
  return NSM_OK;
}

int nsm_host_chunks(nsm_model* m, int* chunks)
{
  if (!m || !chunks) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  *chunks = host_chunk_count(m);
  return NSM_OK;
}

int nsm_compute_internal_force_host(nsm_model* m, const double* displacement, double* internal_force)
{
  if (!m || !displacement || !internal_force) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  NSM_CUDA(cudaSetDevice(m->device));
  if (m->N == 0) return NSM_OK;
  const int K = host_chunk_count(m);
  if (K > 1) {
    if (m->hp_k != K) NSM_CUDA(build_host_pipe(m, K));
    NSM_CUDA(internal_force_pipelined(m, displacement, internal_force, K));
    return read_status(m);  // synchronizes
  }
  const size_t bytes = sizeof(double) * 3 * m->N;
  NSM_CUDA(cudaMemcpyAsync(m->d_stage, displacement, bytes, cudaMemcpyHostToDevice, m->stream));
  NSM_CUDA(nsm::launch_node_aos_to_soa(m->N, m->ld_n, m->d_stage, m->d_u, m->d_uf, m->stream));
  NSM_CUDA(launch_element(m, -1));
  NSM_CUDA(nsm::launch_node_update(node_args(m, -1, -1, 1), m->stream));
  NSM_CUDA(nsm::launch_node_soa_to_aos(m->N, m->ld_n, m->d_f, m->d_stage, m->stream));
  NSM_CUDA(cudaMemcpyAsync(internal_force, m->d_stage, bytes, cudaMemcpyDeviceToHost, m->stream));
  return read_status(m);  // synchronizes
}

int nsm_set_block_material_callback(nsm_model* m, int block, int num_state, nsm_stress_callback fn, void* user)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  if (block < 0 || block >= (int)m->block_cb.size()) return fail(NSM_ERR_INVALID_ARGUMENT, "no such block");
  if (num_state < 0 || num_state > 64) return fail(NSM_ERR_INVALID_ARGUMENT, "0 to 64 state variables per point");
  if (m->S != 1 || m->d_closure) return fail(NSM_ERR_INVALID_ARGUMENT, "block-material callbacks take single-mesh models");
  if (m->closure) return fail(NSM_ERR_INVALID_ARGUMENT, "the model has a learned closure");
  NSM_CUDA(cudaSetDevice(m->device));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  const size_t rec_bytes = m->elem_bytes() * nsm::kIpRecord * 8 * (size_t)m->ld_e;
  if (fn && !m->d_ip_n) {  // the record buffer of step n: a copy of the current records
    NSM_CUDA(cudaMalloc(&m->d_ip_n, rec_bytes));
    NSM_CUDA(cudaMemcpyAsync(m->d_ip_n, m->d_ip, rec_bytes, cudaMemcpyDeviceToDevice, m->stream));
  }
  m->block_cb[block] = fn ? nsm_model::BlockCallback{fn, user, num_state} : nsm_model::BlockCallback{};
  int ns = 0;
  for (const auto& c : m->block_cb)
    if (c.fn && c.num_state > ns) ns = c.num_state;
  if (ns > m->num_state) {  // the state buffers, zero (initial state)
    const size_t sb = sizeof(double) * 8 * (size_t)m->ld_e * ns;
    if (m->d_state) cudaFree(m->d_state);
    if (m->d_state_n) cudaFree(m->d_state_n);
    m->d_state = m->d_state_n = nullptr;
    NSM_CUDA(cudaMalloc(&m->d_state, sb));
    NSM_CUDA(cudaMalloc(&m->d_state_n, sb));
    NSM_CUDA(cudaMemsetAsync(m->d_state, 0, sb, m->stream));
    NSM_CUDA(cudaMemsetAsync(m->d_state_n, 0, sb, m->stream));
    m->num_state = ns;
  }
  // the block's material on the device: computed by the callback, or its own again
  std::vector<nsm::GroupMaterial> mats = m->h_mats;
  for (size_t b = 0; b < mats.size(); b++)
    if (m->block_cb[b].fn) mats[b].model = nsm::kExternal;
  if (m->num_mats == 1) m->model = mats[0].model;
  NSM_CUDA(cudaMemcpyAsync(m->d_mats, mats.data(), sizeof(nsm::GroupMaterial) * mats.size(), cudaMemcpyHostToDevice,
                           m->stream));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);  // the step is no longer the fused one
  m->graphs.clear();
  return NSM_OK;
}

int nsm_get_state_data(nsm_model* m, double* state)
{
  if (!m || !state) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  if (m->num_state == 0 || m->E == 0) return NSM_OK;
  NSM_CUDA(cudaSetDevice(m->device));
  const int ns = m->num_state;
  std::vector<double> planes((size_t)8 * m->ld_e * ns);
  NSM_CUDA(cudaMemcpyAsync(planes.data(), m->d_state, sizeof(double) * planes.size(), cudaMemcpyDeviceToHost,
                           m->stream));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  for (int e = 0; e < m->E; e++)
    for (int p = 0; p < 8; p++)
      for (int k = 0; k < ns; k++) state[((size_t)e * 8 + p) * ns + k] = planes[((size_t)p * m->ld_e + e) * ns + k];
  return NSM_OK;
}

int nsm_get_ip_data(nsm_model* m, double* F, double* sigma)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  if (m->E == 0) return NSM_OK;
  const int is_float = m->precision == NSM_PRECISION_FP64 ? 0 : 1;
  double*   tmp      = nullptr;
  NSM_CUDA(cudaMalloc(&tmp, sizeof(double) * 72 * (size_t)m->E));
  cudaError_t e = cudaSuccess;
  if (F) {
    e = nsm::launch_ip_to_aos(m->E, m->ld_e, m->d_ip, is_float, 0, tmp, m->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(F, tmp, sizeof(double) * 72 * (size_t)m->E, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  }
  if (sigma && e == cudaSuccess) {
    e = nsm::launch_ip_to_aos(m->E, m->ld_e, m->d_ip, is_float, 1, tmp, m->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(sigma, tmp, sizeof(double) * 48 * (size_t)m->E, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  }
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_fail(e, "nsm_get_ip_data");
  return NSM_OK;
}

int nsm_compute_derived_element_data(nsm_model* m, double* volume, double* stress, double* deformation_gradient)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  if (m->E == 0) return NSM_OK;
  const int    is_float = m->precision == NSM_PRECISION_FP64 ? 0 : 1;
  const size_t E        = (size_t)m->E;
  double*      tmp      = nullptr;
  NSM_CUDA(cudaMalloc(&tmp, sizeof(double) * 16 * E));
  cudaError_t e = nsm::launch_derived_element(m->E, m->ld_e, m->d_conn, m->d_X, m->d_u, m->ld_n, m->d_ip, is_float,
                                              tmp, tmp + E, tmp + 7 * E, m->d_status, m->stream);
  if (e == cudaSuccess && volume) e = cudaMemcpyAsync(volume, tmp, sizeof(double) * E, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess && stress)
    e = cudaMemcpyAsync(stress, tmp + E, sizeof(double) * 6 * E, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess && deformation_gradient)
    e = cudaMemcpyAsync(deformation_gradient, tmp + 7 * E, sizeof(double) * 9 * E, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_fail(e, "nsm_compute_derived_element_data");
  return read_status(m);
}

int nsm_get_energies(nsm_model* m, double* kinetic, double* internal)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  NSM_CUDA(nsm::launch_energies(m->N, m->ld_n, m->d_mass, m->d_v, m->E, m->ld_e, m->d_conn, m->d_u, m->d_geo,
                                m->d_elem_group, m->d_mats, m->d_scratch, m->d_out + 2, m->stream));
  double out[2];
  NSM_CUDA(cudaMemcpyAsync(out, m->d_out + 2, sizeof(out), cudaMemcpyDeviceToHost, m->stream));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  if (kinetic) *kinetic = out[0];
  if (internal) *internal = out[1];
  return NSM_OK;
}

int nsm_begin_ensemble(nsm_model* m, double initial_time, const double* final_times, int num_steps,
                       int output_frequency, const double* v_init)
{
  if (!m || !final_times) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  if (num_steps < 0 || output_frequency < 0) return fail(NSM_ERR_INVALID_ARGUMENT, "negative step count");
  for (int g = 0; g < m->S; g++)
    if (final_times[g] < initial_time) return fail(NSM_ERR_INVALID_ARGUMENT, "final time is less than initial time");
  NSM_CUDA(cudaSetDevice(m->device));
  // per-sample schedules as src/integrators/explicit_time_integrator.cc:130-199
  // forms them, laid out [step][sample]
  const int S = m->S;
  m->h_sched.assign((size_t)(num_steps > 0 ? num_steps : 1) * S, StepSched{0, 0, 0, 0, 0});
  m->h_time.assign((size_t)(num_steps + 1), initial_time);
  for (int g = 0; g < S; g++) {
    double t_cur = initial_time, t_prev = initial_time;
    double dt_user = num_steps > 0 ? (final_times[g] - initial_time) / num_steps : 0.0;
    for (int s = 0; s < num_steps; s++) {
      t_prev = t_cur;
      t_cur += dt_user;
      StepSched& q = m->h_sched[(size_t)s * S + g];
      q.delta      = t_cur - t_prev;
      q.half       = 0.5 * q.delta;
      q.time       = t_cur;
      q.is_output  = (output_frequency != 0 && (s % output_frequency == 0 || s == num_steps - 1)) ? 1 : 0;
      if (g == 0) m->h_time[s + 1] = t_cur;
    }
  }
  if (m->d_sched) cudaFree(m->d_sched);
  m->d_sched = nullptr;
  NSM_CUDA(cudaMalloc(&m->d_sched, sizeof(StepSched) * m->h_sched.size()));
  NSM_CUDA(cudaMemcpyAsync(m->d_sched, m->h_sched.data(), sizeof(StepSched) * m->h_sched.size(),
                           cudaMemcpyHostToDevice, m->stream));
  // graphs hold the schedule pointer: rebuild them
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);
  m->graphs.clear();
  NSM_CUDA(cudaMemsetAsync(m->d_step_base, 0, sizeof(int), m->stream));
  const size_t nb = sizeof(double) * 3 * m->ld_n;
  NSM_CUDA(cudaMemsetAsync(m->d_u, 0, nb, m->stream));
  NSM_CUDA(sync_uf(m));
  NSM_CUDA(cudaMemsetAsync(m->d_v, 0, nb, m->stream));
  NSM_CUDA(cudaMemsetAsync(m->d_a, 0, nb, m->stream));
  NSM_CUDA(cudaMemsetAsync(m->d_f, 0, nb, m->stream));
  if (m->d_ip_n) {  // the split step's element data: F = I, sigma = 0 at both levels, zero state
    const size_t rec_bytes = m->elem_bytes() * nsm::kIpRecord * 8 * (size_t)m->ld_e;
    const int    is_float  = m->precision == NSM_PRECISION_FP64 ? 0 : 1;
    for (void* rec : {m->d_ip, m->d_ip_n}) {
      NSM_CUDA(cudaMemsetAsync(rec, 0, rec_bytes, m->stream));
      NSM_CUDA(nsm::launch_ip_identity(m->E, m->ld_e, rec, is_float, m->stream));
    }
    if (m->num_state > 0)
      for (double* st : {m->d_state, m->d_state_n})
        NSM_CUDA(cudaMemsetAsync(st, 0, sizeof(double) * 8 * (size_t)m->ld_e * m->num_state, m->stream));
  }
  int r = nsm_apply_initial_conditions(m);
  if (r) return r;
  if (v_init) {
    r = nsm_set_node_field(m, NSM_FIELD_VELOCITY, v_init);
    if (r) return r;
  }
  r = nsm_apply_kinematic_conditions(m, initial_time, initial_time);
  if (r) return r;
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  m->num_steps  = num_steps;
  m->steps_done = 0;
  m->t0         = initial_time;
  m->begun      = true;
  return NSM_OK;
}

int nsm_begin(nsm_model* m, double initial_time, double final_time, int num_steps, int output_frequency,
              const double* v_init)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  std::vector<double> ft(m->S, final_time);
  return nsm_begin_ensemble(m, initial_time, ft.data(), num_steps, output_frequency, v_init);
}

int nsm_advance(nsm_model* m, int num_steps)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  if (!m->begun) return fail(NSM_ERR_STATE, "nsm_advance before nsm_begin");
  if (num_steps < 0 || m->steps_done + num_steps > m->num_steps)
    return fail(NSM_ERR_INVALID_ARGUMENT, "advance past the end of the schedule");
  NSM_CUDA(cudaSetDevice(m->device));
  int r0 = upload_bcs(m);
  if (r0) return r0;
  if (has_callbacks(m)) {  // one step at a time without graphs: each callback sees its step's times
    for (; num_steps > 0; num_steps--) {
      m->cb_failed  = false;
      cudaError_t e = enqueue_chunk(m, 1, m->profiling);
      if (m->cb_failed) return fail(NSM_ERR_STATE, "a block-material callback failed");
      NSM_CUDA(e);
      m->steps_done += 1;
    }
    return NSM_OK;
  }
  while (num_steps > 0) {
    int K = num_steps < m->graph_steps ? num_steps : m->graph_steps;
    if (m->profiling) {
      NSM_CUDA(enqueue_chunk(m, K, true));
    } else {
      cudaGraphExec_t exec;
      int             r = get_graph(m, K, &exec);
      if (r) return r;
      NSM_CUDA(cudaGraphLaunch(exec, m->stream));
    }
    m->steps_done += K;
    num_steps -= K;
  }
  return NSM_OK;
}

int nsm_advance_timed(nsm_model* m, int num_steps, double* device_ms)
{
  if (!m || !device_ms) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  NSM_CUDA(cudaSetDevice(m->device));
  cudaEvent_t a, b;
  NSM_CUDA(cudaEventCreate(&a));
  NSM_CUDA(cudaEventCreate(&b));
  NSM_CUDA(cudaEventRecord(a, m->stream));
  int r = nsm_advance(m, num_steps);
  cudaEventRecord(b, m->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float       ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (r) return r;
  if (e != cudaSuccess) return cuda_fail(e, "nsm_advance_timed");
  *device_ms = ms;
  return read_status(m);
}

int nsm_progress(nsm_model* m, int* steps_done, double* time_current)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  if (steps_done) *steps_done = m->steps_done;
  if (time_current) *time_current = m->begun ? m->h_time[m->steps_done] : 0.0;
  return NSM_OK;
}

int nsm_synchronize(nsm_model* m)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  return NSM_OK;
}

int nsm_check_status(nsm_model* m)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  return read_status(m);
}

int nsm_time_kernels(nsm_model* m, int repeats, double* element_ms, double* node_ms)
{
  if (!m || repeats <= 0) return fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  NSM_CUDA(cudaSetDevice(m->device));
  cudaEvent_t a, b, c;
  NSM_CUDA(cudaEventCreate(&a));
  NSM_CUDA(cudaEventCreate(&b));
  NSM_CUDA(cudaEventCreate(&c));
  cudaEventRecord(a, m->stream);
  for (int r = 0; r < repeats; r++) NSM_CUDA(launch_element(m, -1));
  cudaEventRecord(b, m->stream);
  for (int r = 0; r < repeats; r++) NSM_CUDA(nsm::launch_node_update(node_args(m, -1, -1, 1), m->stream));
  cudaEventRecord(c, m->stream);
  NSM_CUDA(cudaEventSynchronize(c));
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, a, b);
  cudaEventElapsedTime(&ms2, b, c);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaEventDestroy(c);
  if (element_ms) *element_ms = ms1 / repeats;
  if (node_ms) *node_ms = ms2 / repeats;
  return read_status(m);
}

// Element-kernel launch shapes the autotuner tries: elements per block; one
// pass (one thread per element; blocks_per_sm > 0 then bounds the registers
// so that many 128-thread blocks fit an SM, FP64 form) or a persistent grid of
// blocks per SM walking the elements of all samples; and, in the FP32 form,
// the persistent grid with the nodal values staged one element ahead.
// Shapes a form does not have fall back to its plain launch.
static const nsm::ElementLaunch kLaunchCandidates[] = {
    {128, 0, 0, 0}, {64, 0, 0, 0},  {128, 1, 1, 0}, {128, 1, 2, 0}, {128, 1, 4, 0}, {64, 1, 2, 0},
    {64, 1, 4, 0},  {64, 1, 8, 0},  {128, 0, 3, 0}, {128, 1, 3, 1}, {64, 1, 6, 1},
};
static const int kNumLaunchCandidates = sizeof(kLaunchCandidates) / sizeof(kLaunchCandidates[0]);

int nsm_launch_candidate_times(nsm_model* m, int repeats, double* ms, int capacity, int* count)
{
  if (!m || repeats <= 0 || (capacity > 0 && !ms)) return fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  if (count) *count = kNumLaunchCandidates;
  NSM_CUDA(cudaSetDevice(m->device));
  const nsm::ElementLaunch keep = m->elaunch;
  cudaEvent_t              a, b;
  NSM_CUDA(cudaEventCreate(&a));
  NSM_CUDA(cudaEventCreate(&b));
  cudaError_t err = cudaSuccess;
  for (int c = 0; c < kNumLaunchCandidates && c < capacity && err == cudaSuccess; c++) {
    m->elaunch = kLaunchCandidates[c];
    err        = launch_element(m, -1);  // warm
    if (err == cudaSuccess) err = cudaEventRecord(a, m->stream);
    for (int r = 0; r < repeats && err == cudaSuccess; r++) err = launch_element(m, -1);
    if (err == cudaSuccess) err = cudaEventRecord(b, m->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(b);
    float t = 0;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, a, b);
    ms[c] = t / repeats;
  }
  m->elaunch = keep;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  NSM_CUDA(err);
  return read_status(m);
}

int nsm_set_launch_candidate(nsm_model* m, int candidate)
{
  if (!m || candidate < 0 || candidate >= kNumLaunchCandidates)
    return fail(NSM_ERR_INVALID_ARGUMENT, "invalid launch candidate");
  m->elaunch = kLaunchCandidates[candidate];
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);  // captured with the old shape
  m->graphs.clear();
  return NSM_OK;
}

int nsm_autotune(nsm_model* m, int repeats, int* chosen, double* best_ms)
{
  if (!m || repeats <= 0) return fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  double t[kNumLaunchCandidates];
  int    rc = nsm_launch_candidate_times(m, repeats, t, kNumLaunchCandidates, nullptr);
  if (rc != NSM_OK) return rc;
  int best = 0;
  for (int c = 1; c < kNumLaunchCandidates; c++)
    if (t[c] < t[best]) best = c;
  m->elaunch = kLaunchCandidates[best];
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);  // captured with the old shape
  m->graphs.clear();
  if (chosen) *chosen = best;
  if (best_ms) *best_ms = t[best];
  return NSM_OK;
}

int nsm_set_mlp_closure(nsm_model* m, nsm_mlp* closure)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  if (closure) {
    if (m->precision != NSM_PRECISION_FP32_MIXED) return fail(NSM_ERR_INVALID_ARGUMENT, "the learned closure runs in the FP32-mixed form");
    if (m->S != 1 || m->num_mats != 1 || m->model != NSM_MATERIAL_NEOHOOKEAN)
      return fail(NSM_ERR_INVALID_ARGUMENT, "the learned closure is trained for one neo-Hookean material");
    double K = 0, G = 0;
    nsm::mlp::MlpElementArgs ma;
    nsm::mlp::element_args(closure, &ma, &K, &G);
    if (K != m->K || G != m->G) return fail(NSM_ERR_INVALID_ARGUMENT, "closure trained for another material");
  }
  NSM_CUDA(cudaSetDevice(m->device));
  if (!m->d_fallbacks) {
    NSM_CUDA(cudaMalloc(&m->d_fallbacks, sizeof(unsigned long long)));
    NSM_CUDA(cudaMemsetAsync(m->d_fallbacks, 0, sizeof(unsigned long long), m->stream));
  }
  if (closure && !m->d_closure_geo) {  // the reference geometry of every point, once
    NSM_CUDA(cudaMalloc(&m->d_closure_geo, sizeof(float) * 96 * (size_t)m->ld_e));
    NSM_CUDA(nsm::mlp::launch_closure_geometry(element_args(m, -1), m->d_closure_geo, m->stream));
  }
  m->closure = closure;
  for (auto& g : m->graphs) cudaGraphExecDestroy(g.second);
  m->graphs.clear();
  return NSM_OK;
}

int nsm_closure_fallbacks(nsm_model* m, unsigned long long* count)
{
  if (!m || !count) return fail(NSM_ERR_INVALID_ARGUMENT, "null argument");
  *count = 0;
  if (!m->d_fallbacks) return NSM_OK;
  NSM_CUDA(cudaMemcpyAsync(count, m->d_fallbacks, sizeof(unsigned long long), cudaMemcpyDeviceToHost, m->stream));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  return NSM_OK;
}

int nsm_launches_per_advance(nsm_model* m, int num_steps)
{
  if (!m || num_steps < 0) return -1;
  int launches = 0;
  while (num_steps > 0) {
    int K = num_steps < m->graph_steps ? num_steps : m->graph_steps;
    launches += 2 + 2 * K;
    num_steps -= K;
  }
  return launches;
}

// Profiling mode: nsm_advance launches without graphs and brackets every
// element and node kernel with CUDA events on the model's stream.
int nsm_set_profiling(nsm_model* m, int enable)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  m->profiling    = enable != 0;
  m->ev_elem_used = 0;
  m->ev_node_used = 0;
  return NSM_OK;
}

int nsm_get_profile(nsm_model* m, double* element_ms_total, int* element_launches, double* node_ms_total,
                    int* node_launches)
{
  if (!m) return fail(NSM_ERR_INVALID_ARGUMENT, "null model");
  NSM_CUDA(cudaSetDevice(m->device));
  NSM_CUDA(cudaStreamSynchronize(m->stream));
  double te = 0, tn = 0;
  for (size_t i = 0; i < m->ev_elem_used; i++) {
    float ms = 0;
    NSM_CUDA(cudaEventElapsedTime(&ms, m->ev_elem[i].first, m->ev_elem[i].second));
    te += ms;
  }
  for (size_t i = 0; i < m->ev_node_used; i++) {
    float ms = 0;
    NSM_CUDA(cudaEventElapsedTime(&ms, m->ev_node[i].first, m->ev_node[i].second));
    tn += ms;
  }
  if (element_ms_total) *element_ms_total = te;
  if (element_launches) *element_launches = (int)m->ev_elem_used;
  if (node_ms_total) *node_ms_total = tn;
  if (node_launches) *node_launches = (int)m->ev_node_used;
  m->ev_elem_used = 0;
  m->ev_node_used = 0;
  return NSM_OK;
}

int nsm_device_sm_count(int device, int* count)
{
  if (!count) return fail(NSM_ERR_INVALID_ARGUMENT, "null count");
  cudaError_t e = cudaDeviceGetAttribute(count, cudaDevAttrMultiProcessorCount, device);
  return e == cudaSuccess ? NSM_OK : cuda_fail(e, "cudaDeviceGetAttribute");
}

void* nsm_host_alloc(size_t bytes)
{
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    g_error = "cudaMallocHost failed";
    return nullptr;
  }
  return p;
}

void nsm_host_free(void* p)
{
  if (p) cudaFreeHost(p);
}

}  // extern "C"
