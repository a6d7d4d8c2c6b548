/* CPU oracle for the explicit hex8 / neo-Hookean step: a plain-C restatement
 * of NimbleSM's host algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load this library, and only as the
 * checker or as the timed CPU baseline.  The product (nimblesm_gb300) never
 * links or calls it.
 *
 * Every routine restates the reference operation by operation, in the same
 * order, so that with -ffp-contract=off it reproduces the reference's
 * doubles bit for bit (pinned against the reference itself, compiled from its
 * sources into oracle/_ref, and against its gold files).
 */
#ifndef NSM_ORACLE_H
#define NSM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary-condition kinds, as BoundaryCondition::BC_TYPE
 * (src/nimble_boundary_condition.h). */
enum { NSM_ORACLE_INITIAL_VELOCITY = 0, NSM_ORACLE_PRESCRIBED_VELOCITY = 1, NSM_ORACLE_PRESCRIBED_DISPLACEMENT = 2 };

typedef struct nsm_oracle_model {
  int           num_nodes;
  int           num_elem;
  const double* coords; /* [N][3] reference coordinates */
  const int*    conn;   /* [E][8] 0-based, reference corner order */
  double        density, bulk_modulus, shear_modulus;
  /* Boundary conditions in the order of the input deck; each applies a
   * constant magnitude to one component over a node list. */
  int           num_bcs;
  const int*    bc_kind;      /* [num_bcs] */
  const int*    bc_component; /* [num_bcs] 0,1,2 */
  const double* bc_value;     /* [num_bcs] */
  const int*    bc_ptr;       /* [num_bcs+1] offsets into bc_nodes */
  const int*    bc_nodes;
  /* Material model of the single material (NSM_ORACLE_NEOHOOKEAN /
   * NSM_ORACLE_ELASTIC, the names of src/nimble_material_factory.cc:57-70).
   * With num_blocks > 1 each element takes the material of its block
   * (elem_block [E], elements ordered by block) and the single-material
   * fields above are unused. */
  int           material_model;
  int           num_blocks;
  const int*    elem_block;    /* [E] */
  const int*    block_model;   /* [num_blocks] */
  const double* block_density; /* [num_blocks] */
  const double* block_bulk;    /* [num_blocks] */
  const double* block_shear;   /* [num_blocks] */
} nsm_oracle_model;

#define NSM_ORACLE_NEOHOOKEAN 0
#define NSM_ORACLE_ELASTIC 1

/* Results of a run.  Every pointer may be NULL. */
typedef struct nsm_oracle_result {
  double* u;      /* [N][3] displacement */
  double* v;      /* [N][3] velocity */
  double* a;      /* [N][3] acceleration */
  double* f_int;  /* [N][3] internal force */
  double* F;      /* [E][8][9] deformation gradient, reference component order */
  double* sigma;  /* [E][8][6] Cauchy stress, reference component order */
  double* mass;   /* [N] lumped mass */
  double  dt_crit;
  double  kinetic_energy;
  double  internal_energy;
  double  loop_seconds;
} nsm_oracle_result;

/* Shape-function tables at the 2x2x2 Gauss points (src/nimble_element.cc:55-171):
 * values [ip][node], derivatives [ip][node][3]. */
void nsm_oracle_shape_tables(double* values, double* derivatives);

/* Deformation gradients of one element (src/nimble_element.h:430-502 through
 * src/nimble_element.cc:333-351).  X, x: [8][3] reference / current coords. */
void nsm_oracle_deformation_gradients(const double* X, const double* x, double* F);

/* Neo-Hookean Cauchy stress of n points (src/nimble_material.cc:226-310). */
void nsm_oracle_stress(int n, const double* F, double bulk_modulus, double shear_modulus, double* sigma);

/* Cauchy stress of n points of the given material model (NSM_ORACLE_*):
 * neo-Hookean as above, or ElasticMaterial::GetStress
 * (src/nimble_material.cc:67-126). */
void nsm_oracle_stress_model(
    int model, int n, const double* F, double bulk_modulus, double shear_modulus, double* sigma);

/* Nodal forces of one element (src/nimble_element.h:540-625 through
 * src/nimble_element.cc:457-472).  x [8][3] current coords, sigma [8][6]. */
void nsm_oracle_nodal_forces(const double* x, const double* sigma, double* f);

/* One element end to end, as the block functor (src/nimble_block.cc:278-385). */
void nsm_oracle_element(
    const double* X, const double* u, double bulk_modulus, double shear_modulus, double* F, double* sigma, double* f);

/* Volume average of nq point quantities of one element (src/nimble_element.cc:262-282,
 * src/nimble_element.h:343-392): x [8][3] current coordinates, q [8][nq]
 * (nq <= 32); volume and avg [nq] out. */
void nsm_oracle_volume_average(const double* x, int nq, const double* q, double* volume, double* avg);

/* Lumped mass (src/nimble_model_data.cc:495-530, src/nimble_block.cc:110-146,
 * src/nimble_element.cc:173-193) and critical time step
 * (src/nimble_block_base.cc:51-84, src/nimble_element.cc:221-260). */
void   nsm_oracle_lumped_mass(const nsm_oracle_model* m, double* mass);
double nsm_oracle_critical_time_step(const nsm_oracle_model* m);

/* The reference's UQ mode (src/uq/nimble_uq_model_data.cc:55-248,
 * src/uq/nimble_uq.cc:270-345): the nominal trajectory of m, num_exact
 * trajectories with moduli exact_bulk / exact_shear [num_exact][blocks], and
 * num_approx trajectories driven by the closure coef [num_approx][num_exact+1]
 * (nominal first).  v_init (nullable) is every trajectory's initial velocity.
 * Records after every output step (the last step when output_frequency is 0),
 * at most max_outputs: nominal u, v, f [T][N][3]; samples su, sv, sf
 * [T][num_exact + num_approx][N][3], exact first.  0, or -1 on an inverted
 * element. */
int nsm_oracle_run_uq(const nsm_oracle_model* m, int num_exact, const double* exact_bulk, const double* exact_shear,
                      int num_approx, const double* coef, double final_time, int num_steps, int output_frequency,
                      const double* v_init, int num_threads, int max_outputs, double* out_u, double* out_v,
                      double* out_f, double* out_su, double* out_sv, double* out_sf, int* out_num_outputs);

/* Derived element output over a model (src/nimble_block.cc:438-497): u [N][3],
 * sigma [E][8][6], F [E][8][9] -> volume [E], avg_sigma [E][6], avg_F [E][9]. */
void nsm_oracle_derived_element_data(const nsm_oracle_model* m, const double* u, const double* sigma, const double* F,
                                     double* volume, double* avg_sigma, double* avg_F);

/* Strain energy density W(F) whose Cauchy stress is the reference's
 * neo-Hookean stress: W = K/4 (J^2-1) - K/2 ln J + G/2 (J^{-2/3} tr(F F^T) - 3).
 * Not in the reference; defined here for the energy balance. */
double nsm_oracle_energy_density(const double* F, double bulk_modulus, double shear_modulus);

/* The explicit loop (src/integrators/explicit_time_integrator.cc:123-278):
 * lumped mass, critical time step, initial and kinematic conditions, then
 * num_steps central-difference steps with dt = final_time / num_steps.
 * v_init (nullable, [N][3]) overwrites the velocity after the initial
 * conditions and before ApplyKinematicConditions(0,0).  output_frequency as in
 * the input deck (0 = no output steps).  num_threads > 1 parallelises the
 * element loop with OpenMP; the assembly is a node-ordered gather that adds
 * element contributions in increasing element order, the same order as the
 * reference's serial loop (src/nimble_block.cc:373-383, :434), so the result
 * does not depend on the thread count.  Returns 0, or -1 on a non-positive
 * Jacobian (the reference aborts there, src/nimble_utils.h:1243-1255). */
int nsm_oracle_run(
    const nsm_oracle_model* m,
    double                  final_time,
    int                     num_steps,
    int                     output_frequency,
    const double*           v_init,
    int                     num_threads,
    nsm_oracle_result*      out);

/* Same step loop, but starting from a given state (u, v, a; all [N][3]) at
 * time t0 with a fixed user time step; used for bounded timing samples. */
int nsm_oracle_continue(
    const nsm_oracle_model* m,
    double                  t0,
    double                  dt,
    int                     num_steps,
    int                     num_threads,
    double*                 u,
    double*                 v,
    double*                 a,
    double*                 loop_seconds);

/* Extended-precision stress of displacement u at the points of `num` listed
 * elements -> sigma [num][8][6]: the accuracy yardstick (see nsm_oracle.c). */
void nsm_oracle_stress_exact(const nsm_oracle_model* m, const double* u, int num, const int* elems, double* sigma);

/* Stateful form of the same loop, for reading intermediate states. */
typedef struct nsm_oracle nsm_oracle;
nsm_oracle* nsm_oracle_create(const nsm_oracle_model* m, int num_threads); /* lumped mass, dt_crit */
void        nsm_oracle_destroy(nsm_oracle* o);
double      nsm_oracle_dt_crit(const nsm_oracle* o);
void        nsm_oracle_begin(nsm_oracle* o, double final_time, int num_steps, int output_frequency, const double* v_init);
int         nsm_oracle_advance(nsm_oracle* o, int k, double* loop_seconds); /* next k steps of the schedule */
double      nsm_oracle_time(const nsm_oracle* o);
void        nsm_oracle_get_state(const nsm_oracle* o, double* u, double* v, double* a, double* f_int, double* F,
                                 double* sigma, double* mass);
/* The internal force of displacement u [N][3] alone (ModelData::ComputeInternalForce,
 * src/nimble_model_data.cc:620-667) into f_int [N][3]; F and sigma of every
 * point are kept for nsm_oracle_get_state.  0, or -1 on a non-positive Jacobian. */
int         nsm_oracle_internal_force(nsm_oracle* o, const double* u, double* f_int);
void        nsm_oracle_set_state(nsm_oracle* o, const double* u, const double* v, const double* a);
void        nsm_oracle_energies(const nsm_oracle* o, double* kinetic, double* internal);

#ifdef __cplusplus
}
#endif
#endif
