/* dg3d: GB300-native DG right-hand side and SSP-RK3 time loop for 3DDG.
 *
 * C ABI of libdg3d.so.  Plain C types only (no CUDA or C++ types), int status
 * returns (0 = success, negative = error; dg_last_error() has the message),
 * caller-owned host buffers, library-owned device buffers.  One handle per
 * host thread.  All stepping is stream-ordered on the handle's CUDA stream.
 *
 * The reference (drewalan/3DDG) has no plugin or FFI layer: its hot path is the
 * C++ class surface that main() drives (cppsrc/driver.cpp:199-278).  Each
 * entry point below names the reference interface it replaces; the C++ facade
 * classes Grid/Block/Element/Basis in this package (csrc/host/) keep the
 * reference's signatures and call these entry points.
 */
#ifndef DG3D_H
#define DG3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DG_OK 0
#define DG_ERR_INVALID (-1)   /* bad argument or parameter */
#define DG_ERR_CUDA (-2)      /* CUDA runtime error */
#define DG_ERR_NOMEM (-3)     /* device allocation refused or over budget */
#define DG_ERR_IO (-4)        /* file could not be opened, read or written */
#define DG_ERR_STATE (-5)     /* call not valid in the handle's current state */

#define DG_PRECISION_FP64 64  /* the plain method: FP64 fields, fluxes, stages */
#define DG_PRECISION_FP32 32  /* FP32 fields/fluxes, Kahan-compensated update */

/* Simulation parameters.  Field names and meanings follow the reference's
 * parameter file keys (parameters1.txt; parsed at cppsrc/driver.cpp:139-186),
 * the Grid constructor arguments (cppsrc/Grid.h:33) and struct BCParam
 * (cppsrc/BCParam.h:13-36). */
typedef struct dg_params {
    int order;                 /* ORDER: polynomial order N (nodes per line N+1), 1..7 */
    int num_blocks[3];         /* NUM_BLOCKS */
    int num_elements[3];       /* NUM_ELEMENTS, per block */
    double elem_width[3];      /* ELEMENT_WIDTH */
    double corner[3];          /* STARTING_CORNER */
    double rho0;               /* RHO0 */
    double c0;                 /* C0 */
    double b_over_a;           /* B_OVER_A (0 selects the linear mass flux) */
    double diff_const;         /* DIFF_CONST */
    int eval_advect;           /* EVALUATE_ADVECTION */
    int eval_diff;             /* EVALUATE_DIFFUSION */
    int eval_sponge;           /* EVALUATE_SPONGE */
    int periodic[3];           /* BC_IS_PERIODIC */
    double sigma_max;          /* BC_SIGMA_MAX */
    int sponge_width[6];       /* BC_SPONGE_WIDTH: -X +X -Y +Y -Z +Z */
    int ic_gauss[3];           /* IC_X_GAUSS, IC_Y_GAUSS, IC_Z_GAUSS */
    double ic_drho_amp;        /* IC_DRHO_AMPLITUDE */
    double ic_v_amp[3];        /* IC_VX/VY/VZ_AMPLITUDE */
    double ic_sigma;           /* IC_SIGMA (inverse square length) */
    double ic_center[3];       /* IC_CENTER_X/Y/Z */
    /* Extensions (not in the reference; defaults reproduce it): */
    int precision;             /* DG_PRECISION_FP64 (default) or DG_PRECISION_FP32 */
    int rk_exact;              /* 0: the reference's RK weights (its stage-3 weights
                                  2.0F/3.0F, 1.0F/3.0F are float literals); 1: exact */
    int lumped_mass;           /* 1: diagonal LGL mass matrix when none is read from file */
    int src_face;              /* tone-burst source face (-X +X -Y +Y -Z +Z = 0..5), -1 none */
    double src_amp;            /* source pressure amplitude */
    double src_freq;           /* centre frequency */
    double src_cycles;         /* cycles under the Hann window */
    double src_phase;          /* phase offset, radians */
    double src_radius;         /* aperture radius about the face centre (<= 0: whole face) */
} dg_params;

typedef struct dg_handle dg_handle;

/* Fill *p with the reference's BCParam defaults (cppsrc/BCParam.cpp:24) and
 * the driver's compiled-in defaults (cppsrc/driver.cpp:48-65). */
int dg_params_default(dg_params* p);

/* Parse a parameter file in the reference's "KEY = values" format; replaces
 * the parser in main() (cppsrc/driver.cpp:129-196).  Keys absent from the file
 * keep the values already in *p.  Driver-only keys are returned through the
 * optional pointers (NULL to ignore).  If log_path is non-NULL the file is
 * echoed there as "Parameters used:\n{\n  <line>\n}\n" like the reference's
 * _log.txt.  Unknown keys produce the reference's warning on stderr. */
int dg_params_parse(const char* path, dg_params* p, double* dt, int* num_substeps,
                    int* num_outsteps, int* freq_terminal, int* bool_file,
                    const char* log_path);

/* Build the mesh, operators and initial condition and upload them; replaces
 * Grid::Grid + Basis::Basis (cppsrc/Grid.h:33, cppsrc/Basis.h:26) and the
 * three Grid copies the driver makes (cppsrc/driver.cpp:199-213).
 * matrix_file / coeff_file: the reference's matrices.txt and
 * hardcoded_coeff.txt (NULL: computed in FP64 from LGL mathematics). */
int dg_create(const dg_params* p, const char* matrix_file, const char* coeff_file,
              dg_handle** out);

/* Release every device and host resource of the handle. */
int dg_destroy(dg_handle* h);

/* Advance nsteps SSP-RK3 steps of size dt; replaces the driver's inner loop
 * around Grid::RK33 (cppsrc/driver.cpp:256-277, cppsrc/Grid.cpp:642-902),
 * including Grid::communicate (cppsrc/Grid.cpp:487-565), which becomes an
 * on-device face gather.  Asynchronous on the handle's stream. */
int dg_step(dg_handle* h, double dt, int nsteps);

/* Wait for all work queued on the handle: its compute stream and the copy
 * streams of the asynchronous transfers. */
int dg_synchronize(dg_handle* h);

/* Node-duplicated global dimensions X = NB_x*E_x*(N+1), Y, Z: the array shape
 * of the reference's HDF5 datasets (cppsrc/HDF5Functions.cpp:160-168). */
int dg_dims(const dg_handle* h, int* X, int* Y, int* Z);

/* Copy the current state to host buffers: drho [X][Y][Z], vel [3][X][Y][Z]
 * (either may be NULL).  Replaces the gather of dumpToHDF5File
 * (cppsrc/HDF5Functions.cpp:173-208).  Synchronous. */
int dg_get_state(dg_handle* h, double* drho, double* vel);

/* Overwrite the current state from host buffers of the same layout.  Boundary
 * exterior values become zero (no initial-condition halo).  Synchronous. */
int dg_set_state(dg_handle* h, const double* drho, const double* vel);

/* Asynchronous forms of dg_set_state / dg_get_state for page-locked (pinned)
 * host buffers (no counterpart in the reference, whose state never leaves the
 * host).  The copies run on the copy engines through double-buffered device
 * staging on two streams of their own, ordered against dg_step through
 * events; an upload is unpacked on a stream of its own into a spare state
 * buffer that is swapped in at its place in the call sequence, and a download
 * is packed on another, so that the upload of the next input and the download
 * of the last result overlap the steps computing between them.
 * dg_get_state_async captures the state at its place in the call sequence.  Host buffers must
 * stay untouched (inputs) or unread (outputs) until dg_synchronize returns.
 * Pageable buffers are rejected with DG_ERR_INVALID. */
int dg_set_state_async(dg_handle* h, const double* drho, const double* vel);
int dg_get_state_async(dg_handle* h, double* drho, double* vel);
/* One RK step followed by dg_get_state_async of its result, in one call (no
 * counterpart in the reference).  In the FP64 path with advection the step's
 * last stage writes its output in host order into the download staging as it
 * writes the state, so no separate pack runs; the bytes are those of dg_step
 * then dg_get_state_async.  Otherwise it is exactly those two calls.  Host
 * buffers: as dg_get_state_async (pinned, unread until dg_synchronize). */
int dg_step_get_state_async(dg_handle* h, double dt, double* drho, double* vel);

/* One evaluation R = L(u) of the semi-discrete right-hand side at the current
 * state (LDG diffusion, advection, sponge; no RK combination) into host
 * buffers of the dg_get_state layout: the per-stage operator sum that
 * Grid::RK33 accumulates into k1 before selfWeightedAdd (cppsrc/Grid.cpp:
 * 655-704).  The state and time are unchanged.  Synchronous. */
int dg_eval_rhs(dg_handle* h, double* drho, double* vel);

/* Size limits of dg_eval_rhs_noalloc's static scratch. */
#define DG_NOALLOC_MAX_NODES 1048576    /* n_elem * NP node slots, NP = (N+1)^3 rounded up to 8 */
#define DG_NOALLOC_MAX_ELEMENTS 131072

/* The evaluation of dg_eval_rhs for callers that cannot allocate device
 * memory (no counterpart in the reference; it exists for hosts that own all
 * device memory through their own pool or arena, or must not allocate at call
 * time, and therefore cannot create a dg_handle).  The caller passes device
 * buffers it owns: d_state (4 FP64 fields drho, u_x, u_y, u_z, element-major:
 * field f, element e, node n at f*n_elem*NP + e*NP + n, node n = (i*K+j)*K+k),
 * d_nbr (n_elem x 6 face table in the order -X +X -Y +Y -Z +Z: a neighbour
 * element index in [0, n_elem), or -1 - slot with slot < 6*n_elem, i.e. a
 * value in [-6*n_elem, -1], for a boundary face, whose exterior state is zero;
 * the table is not checked, and any other entry is undefined behaviour), d_sigma (n_elem sponge sigmas; may be NULL when
 * eval_sponge is 0) and d_rhs (output, same layout as d_state); host mass and
 * stiff are the (N+1)^2 unit-interval matrices of matrices.txt.  FP64 only,
 * order 1..7, at most DG_NOALLOC_MAX_ELEMENTS elements and
 * DG_NOALLOC_MAX_NODES node slots (larger problems are rejected with
 * DG_ERR_INVALID).  Calls no cudaMalloc/cudaFree or other allocating routine:
 * the LDG-gradient scratch is a 27 MiB static device array that every GPU
 * loading this library holds until exit.  The first call on a device looks up
 * that array's address (cudaGetSymbolAddress), so make it before any stream
 * capture; with CUDA's lazy module loading that call is also when the 27 MiB
 * is taken on the device, so a host with a budgeted device arena makes one
 * call per device at start-up, before committing its arena.  The address is
 * kept for the process's life: a cudaDeviceReset while the library is loaded
 * leaves it stale.  Calls share the scratch: calls whose work overlaps on one
 * GPU race.
 * Asynchronous on ``stream`` (a cudaStream_t, NULL = the default stream). */
int dg_eval_rhs_noalloc(const dg_params* p, const double* mass, const double* stiff,
                        const double* d_state, const int* d_nbr, const double* d_sigma,
                        double* d_rhs, int n_elem, void* stream);

/* Node coordinates [3][X][Y][Z] and per-node sponge sigma [X][Y][Z] (either
 * may be NULL); the data of dumpGridToHDF5File (cppsrc/HDF5Functions.cpp:34-142). */
int dg_get_grid(dg_handle* h, double* coords, double* sigma);

/* Simulation time (sum of the dt of every completed step). */
double dg_time(const dg_handle* h);

/* Write the reference's snapshot files for time step ts into folder/raw/:
 * dRho_<b>_<ts>.h5 ("rho" [X][Y][Z] f64 + "time") and vel_<b>_<ts>.h5
 * ("velocity" [3][X][Y][Z] + "time"), one file pair per block b like one MPI
 * rank of the reference (cppsrc/HDF5Functions.cpp:145-247).  grid = 1 adds,
 * and grid = 2 writes only, the coords/ba/diff/rho0/c0 files of
 * dumpGridToHDF5File (cppsrc/HDF5Functions.cpp:34-142).  The state is copied
 * back from the device only here.  Returns 0, or the reference's codes -1..-4
 * for file/dataset failures. */
int dg_write_snapshot(dg_handle* h, const char* folder, int ts, int grid);

/* Write one HDF5 file holding the float64 dataset ``name`` of rank ndim
 * (dims[0..ndim-1], row-major data) and the one-element float64 dataset
 * "time"; replaces hdf5outputScalar / hdf5outputVector
 * (cppsrc/HDF5Functions.cpp:249-397, whose vector form writes [3][X][Y][Z]).
 * Host only.  Returns 0, or -1 when the file cannot be written. */
int dg_hdf5_write(const char* path, const char* name, int ndim, const long long* dims,
                  const double* data, double time);

/* Read the numeric dataset ``name`` of an HDF5 file's root group, converted to
 * float64 in row-major order; replaces the reference's dormant reader
 * hdf5input (cppsrc/HDF5Functions.cpp:398-463; declared in
 * HDF5Functions.h:26, no caller), without libhdf5.  Reads this library's files
 * and the HDF5 library's default-format files: superblock 0/1, symbol-table
 * root group, contiguous or compact layout, no filters, integer or IEEE float.
 * *ndim receives the rank and dims[0..max_ndim-1] the leading dimensions;
 * with data non-NULL the values are copied when they fit in ``capacity``
 * doubles (else -3).  type_class (may be NULL) receives the HDF5 class, 0
 * integer or 1 floating point.  Returns 0, or the reference's codes by failure
 * class: -1 file, -2 dataset (no such name, chunked/filtered layout),
 * -3 dataspace, -4 datatype; dg_last_error() says which.  Host only. */
int dg_hdf5_read(const char* path, const char* name, int max_ndim, long long* dims, int* ndim,
                 double* data, long long capacity, int* type_class);

/* Restart from a snapshot (the use the reference's hdf5input was written for,
 * cppsrc/HDF5Functions.cpp:398-463): read folder/raw/dRho_<b>_<ts>.h5 and
 * vel_<b>_<ts>.h5 of every block, as dg_write_snapshot writes them, into the
 * state (as dg_set_state does: boundary exterior values become zero) and set
 * the simulation time to the files' "time".  An FP64 handle continues
 * bit-identically to the run that wrote the snapshot.  Returns 0, the codes of
 * dg_hdf5_read, or -3 when a file's shape does not match the grid.
 * Synchronous. */
int dg_read_snapshot(dg_handle* h, const char* folder, int ts);

/* Pressure probes (no counterpart in the reference; for focal-axis and
 * harmonic analysis): after every subsequent RK step the pressure
 * p = c0^2 (drho + B/A drho^2 / (2 rho0)) at the node nearest to each of the n
 * points xyz[3*i..3*i+2] is recorded on the device.  Calling it again
 * replaces the probes and clears the record. */
int dg_probe_set(dg_handle* h, int n, const double* xyz);
/* Copy the record: up to max_steps rows of n values (step-major) into p and
 * the time after each recorded step into t (either may be NULL); *steps
 * receives the number of recorded steps.  Synchronous. */
int dg_probe_get(dg_handle* h, double* t, double* p, int max_steps, int* steps);

/* Number of kernel launches issued by this handle since creation (profiling). */
long long dg_launch_count(const dg_handle* h);

/* The cudaStream_t the handle issues all its work on (as void*), so callers
 * can order their own work against it or time it with CUDA events. */
int dg_stream(dg_handle* h, void** stream);

/* Per-kernel statistics for profiling (no reference counterpart; the
 * reference only had gprof).  dg_profile(h, 1) clears the counters and starts
 * bracketing every stage / LDG-gradient kernel launch with CUDA events on the
 * handle's stream; dg_profile(h, 0) stops.  dg_kernel_stats waits for the
 * stream and returns, per kernel kind k (0 = stage kernel, 1 = LDG gradient),
 * the number of launches, their summed event time in ms, and their summed
 * algorithmic DRAM bytes and FP flops (the data each launch must move once and
 * the arithmetic it must do: per node, the fields read and written once, and
 * 2 flops per FMA of the line sums, face fluxes and stage combination). */
int dg_profile(dg_handle* h, int enable);
int dg_kernel_stats(dg_handle* h, int k, long long* launches, double* ms, double* bytes,
                    double* flops);

/* Device pointers of the current state fields (FP64 or FP32 per precision),
 * element-major: field f, element e, node n at base[f] + e*node_stride + n,
 * node n = (i*K + j)*K + k.  For zero-copy integration and benchmarking.
 * Writes through them must be ordered against the library's stream
 * (dg_stream) and made before the next dg_step; to write again after later
 * steps, call dg_state_device again first (the FP64 path caches the volume
 * fluxes of the state between stages, and this call drops that cache).
 * dg_set_state_async swaps in another state buffer: pointers taken before it
 * are stale after it.  The library's stream is made to wait for a pending
 * dg_get_state_async pack of the state, so writes ordered on dg_stream come
 * after it. */
int dg_state_device(dg_handle* h, void* base[4], size_t* node_stride, int* n_elem);

/* ------------------------------------------------------------------------
 * Batched form (no counterpart in the reference, which runs one problem per
 * process): n independent problems of uneven element counts and orders
 * (ORDER 1..5), FP32 fields/fluxes/stages with the Kahan-compensated update,
 * advanced together by persistent kernels per order (one group of problems
 * per branch of a captured CUDA graph).  Problem i takes its own dt[i] and
 * stops after steps[i] steps;
 * its exterior state is zero except the tone-burst source (whole face).
 * Each problem's result is independent of its batch-mates (bitwise).
 * ------------------------------------------------------------------------ */
typedef struct dg_batch dg_batch;
int dg_batch_create(int n, const dg_params* params, const double* dt, const int* steps,
                    const char* matrix_file, const char* coeff_file, dg_batch** out);
int dg_batch_destroy(dg_batch* b);
/* Advance every active problem nsteps steps (asynchronous). */
int dg_batch_step(dg_batch* b, int nsteps);
int dg_batch_synchronize(dg_batch* b);
/* State of problem i in the dg_get_state layout (synchronous). */
int dg_batch_get_state(dg_batch* b, int i, double* drho, double* vel);
/* Node-duplicated dims, completed steps and time of problem i. */
int dg_batch_info(dg_batch* b, int i, int* dims3, long long* steps_done, double* time);
long long dg_batch_total_nodes(const dg_batch* b);
/* Choose the tile size of every order and the persistent grid by timing
 * trial_steps real steps per candidate; the state is restored afterwards.
 * A summary of the choice is written to report (may be NULL). */
int dg_batch_autotune(dg_batch* b, int trial_steps, char* report, size_t report_len);
int dg_batch_stream(dg_batch* b, void** stream);
long long dg_batch_launch_count(const dg_batch* b);

/* ------------------------------------------------------------------------
 * Serving form (no counterpart in the reference): a request loop that admits
 * solves by an HBM budget, keeps their state on the device and batches their
 * RK steps with every other in-flight solve (continuous batching, the batched
 * form's kernels).  Clock: seconds since dg_serve_create.
 * ------------------------------------------------------------------------ */
typedef struct dg_server dg_server;
/* keep_results != 0: copy each finished solve's state back for dg_serve_result. */
int dg_serve_create(size_t hbm_budget_bytes, int keep_results, dg_server** out);
int dg_serve_destroy(dg_server* s);
double dg_serve_clock(const dg_server* s);
/* Queue a solve arriving at arrival_time (server clock; < 0: now).  Rejected
 * with DG_ERR_NOMEM if it alone exceeds the budget. */
int dg_serve_submit(dg_server* s, const dg_params* p, double dt, int steps, double arrival_time,
                    long long* id);
/* One loop iteration: collect the ticks the device has finished (their
 * requests get their completion times and results), admit arrived requests
 * that fit and whose host preparation (mesh tables, operators, staged in
 * page-locked memory by the server's worker thread) is done, enqueue for every
 * in-flight solve the same number of RK steps (one graph replay each): as many
 * as end no in-flight solve early and, while a request is still to arrive, as
 * fit before its arrival by the running estimate of a step's time (at most
 * 64; one while an arrived request waits for its preparation), and enqueue
 * the retirement of the solves these steps complete (result copy, memory back
 * to the server's device memory pool).  Admission and retirement are
 * stream-ordered device work, so the host never synchronises the device for
 * them; it waits only to stay at most two ticks ahead of the device, and
 * drains when nothing is in flight.  dg_serve_submit, dg_serve_result,
 * dg_serve_stats and dg_serve_utilization may be called from any thread
 * (submissions go through an internal queue that the loop drains at each
 * iteration); dg_serve_tick and dg_serve_run from one thread at a time. */
int dg_serve_tick(dg_server* s, int* n_inflight);
/* Run the loop in real time until every submitted request has finished. */
int dg_serve_run(dg_server* s, double max_seconds);
/* Arrival, admission and completion times of a request; its final state when
 * the server keeps results (drho/vel may be NULL).  A request whose host
 * preparation failed is set aside (the loop goes on with the others) and
 * returns that error here. */
int dg_serve_result(dg_server* s, long long id, double* t_arrival, double* t_admit, double* t_done,
                    double* drho, double* vel);
/* Completed requests, p50/p99 latency (s), completed solves per second over
 * the span from the first arrival to the last completion, mean in-flight count. */
int dg_serve_stats(dg_server* s, int* completed, double* p50, double* p99, double* solves_per_s,
                   double* mean_inflight);
/* Device time spent in RK steps (CUDA events around each tick's steps), the
 * span from the first arrival to the last completion, and the DOF-stage
 * updates performed (4 fields x nodes x 3 stages x steps, summed over every
 * solve); busy / span is the device's busy fraction over the trace. */
int dg_serve_utilization(dg_server* s, double* gpu_busy_s, double* span_s, double* dof_stage_updates);

/* Last error message of this thread ("" if none). */
const char* dg_last_error(void);

/* Write hardcoded_coeff.txt, hardcoded_coeff2.txt (point counts 1..kmax) and
 * matrices.txt (orders 1..kmax-1) into folder, in the formats the reference
 * reads (cppsrc/Basis.cpp:74-237, cppsrc/Grid.cpp:920-989). */
int dg_write_basis_files(const char* folder, int kmax, int lumped_mass);

/* Unit-interval operators of one order as used on the device: mass, stiff,
 * deriv (D = M^-1 S) each (N+1)^2 row-major, lift0/liftN (N+1), zeros (N+1). */
int dg_line_operators(int order, int lumped_mass, const char* matrix_file,
                      const char* coeff_file, double* mass, double* stiff,
                      double* deriv, double* lift0, double* liftN, double* zeros);

#ifdef __cplusplus
}
#endif
#endif /* DG3D_H */
