/* CPU oracle for the DG right-hand side and SSP-RK3 time loop of 3DDG.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference's algorithm, used by the tests, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg as the checker.  The product never links it.
 *
 * Data layout follows the reference: every block of E_x*E_y*E_z elements
 * carries a one-element halo ring (cppsrc/Block.cpp:167-247); every element
 * holds (N+1)^3 nodes with 7 fields {rho, u0, u1, u2, q0, q1, q2}
 * (cppsrc/Node.h:77-80).  Multi-block meshes are restated as one block of the
 * global size: the reference's face exchange (cppsrc/Grid.cpp:487-565) makes
 * every inter-block halo equal to the neighbour block's face layer before each
 * operator, which is exactly what a single block's interior neighbours give.
 */
#ifndef DG_ORACLE_H
#define DG_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct dgo_params {
    int order;               /* ORDER */
    int num_blocks[3];       /* NUM_BLOCKS */
    int num_elements[3];     /* NUM_ELEMENTS (per block) */
    double elem_width[3];    /* ELEMENT_WIDTH */
    double corner[3];        /* STARTING_CORNER */
    double rho0, c0, b_over_a, diff_const;
    int eval_advect, eval_diff, eval_sponge;
    int periodic[3];         /* BC_IS_PERIODIC */
    double sigma_max;        /* BC_SIGMA_MAX */
    int sponge_width[6];     /* BC_SPONGE_WIDTH: -X +X -Y +Y -Z +Z */
    int ic_gauss[3];         /* IC_X/Y/Z_GAUSS */
    double ic_drho_amp, ic_v_amp[3], ic_sigma, ic_center[3];
    /* SSP-RK3 weights: 0 = the reference's literals (its stage-3 weights
       2.0F/3.0F and 1.0F/3.0F are float-rounded even in an FP64 build),
       1 = exact 2/3 and 1/3. */
    int rk_exact;
    /* Tone-burst boundary source (absent from the reference; this package's
       definition): face index in -X +X -Y +Y -Z +Z order, or -1 for none. */
    int src_face;
    double src_amp, src_freq, src_cycles, src_phase, src_radius;
} dgo_params;

typedef struct dgo_sim dgo_sim;

/* mass, stiff: (N+1)x(N+1) row-major unit-interval matrices (matrices.txt);
   zeros: N+1 LGL zeros on [-1, 1] (hardcoded_coeff.txt).  NULL on error. */
dgo_sim* dgo_create(const dgo_params* p, const double* mass, const double* stiff,
                    const double* zeros);
void dgo_destroy(dgo_sim* s);
/* Advance nsteps RK33 steps of size dt, swapping grids like cppsrc/driver.cpp:271-275. */
void dgo_run(dgo_sim* s, double dt, int nsteps);
/* Node-duplicated interior state, X = E_x*NB_x*(N+1) ...: rho [X][Y][Z], vel [3][X][Y][Z]. */
void dgo_get_state(const dgo_sim* s, double* rho, double* vel);
/* Overwrite the interior state; every halo becomes zero (no stale IC halos). */
void dgo_set_state(dgo_sim* s, const double* rho, const double* vel);
/* Node coordinates [3][X][Y][Z] and per-node sponge sigma [X][Y][Z]. */
void dgo_get_coords(const dgo_sim* s, double* coords, double* sigma);
double dgo_time(const dgo_sim* s);
/* One right-hand-side evaluation L(u) of the current state (diffusion,
   advection, sponge; no RK combination) into rho/vel node-duplicated arrays. */
void dgo_rhs(dgo_sim* s, double* rho, double* vel);

#ifdef __cplusplus
}
#endif
#endif
