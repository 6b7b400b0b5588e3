/*
 * ffea_gpu.h -- C ABI of the GB300 (sm_103a) FFEA blob-step engine.
 *
 * Drop-in for FFEA's per-timestep blob update (RSE-Sheffield/ffea_ci_demo,
 * FFEA 2.7.2). The reference has no C ABI: its path sits behind the C++
 * classes Blob (include/Blob.h:94-718) and Solver (include/Solver.h:31-52).
 * Each entry point below names the reference member it replaces.
 *
 * Conventions
 *  - Every call returns an int status (FFEA_GPU_OK or an FFEA_GPU_E* code);
 *    nothing throws across the ABI and device code never traps.
 *  - Host arrays are caller-owned and copied; device memory is owned by the
 *    handle. Calls on one handle are not thread-safe.
 *  - Units are FFEA's meso units (include/dimensions.h:30-41) unless a
 *    function says SI; helpers convert exactly as the reference loaders do.
 *  - Node arrays cover every node of the 10-node ("quadratic") topology in
 *    the reference's node order; the device carries vertex nodes only and
 *    rebuilds edge-midpoint nodes when state is read back, as the reference
 *    does every step (tetra_element_linear::linearise_element).
 */
#ifndef FFEA_GPU_H
#define FFEA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FFEA_GPU_OK 0
#define FFEA_GPU_EINVERTED 1 /* an element inverted (Blob::update_internal_forces, src/Blob.cpp:484-490) */
#define FFEA_GPU_ECGMAXIT 2  /* CG hit max_iterations_cg (NoMassCGSolver::solve, src/NoMassCGSolver.cpp:187) */
#define FFEA_GPU_EINPUT 3    /* invalid argument, mesh or parameter */
#define FFEA_GPU_ENOMEM 4    /* device or host allocation failed */
#define FFEA_GPU_ECUDA 5     /* CUDA runtime error or extension built for another GPU */
#define FFEA_GPU_ENAN 6      /* non-finite solver output (FP64 path: e.g. an exactly zero right-hand side, as the
                                reference's alpha = 0/0; the mixed path returns x = 0 for it) */
#define FFEA_GPU_ETIMEOUT 7  /* a bounded device-side wait gave up */
#define FFEA_GPU_EFILE 8     /* structure file missing or malformed (FFEAFileException) */

/* solvers: the `solver` keyword of a .ffea <blob> block (src/World.cpp:2601-2627) */
#define FFEA_GPU_NOMASS_CG 0  /* "CG_nomass"  -> NoMassCGSolver */
#define FFEA_GPU_CG 1         /* "CG"         -> ConjugateGradientSolver (consistent mass) */
#define FFEA_GPU_MASSLUMPED 2 /* "masslumped" -> MassLumpedSolver */

/* arithmetic of the step */
#define FFEA_GPU_FP64 0  /* every operation in FP64, in the reference's evaluation order */
#define FFEA_GPU_MIXED 1 /* FP32 element stress, noise scaling, matrix and SpMV; FP64 dot products,
                            residual norms, near-degenerate Jacobians and the position accumulator */

/* the hot-path fields of SimulationParams (include/SimulationParams.h:75-211), meso units */
typedef struct ffea_gpu_params {
    double dt;          /* time step */
    double kT;          /* thermal energy */
    double epsilon2;    /* CG stop: |r|^2/|f|^2 < epsilon2 (the script's epsilon, squared) */
    double stokes_visc; /* medium viscosity for Stokes drag */
    int max_iterations_cg;
    int calc_noise;   /* 1: thermal fluctuating stress (and Stokes noise) */
    int calc_stokes;  /* 1: Stokes drag 6 pi eta r on every node */
    int solver;       /* FFEA_GPU_NOMASS_CG / FFEA_GPU_CG / FFEA_GPU_MASSLUMPED */
    int precision;    /* FFEA_GPU_FP64 / FFEA_GPU_MIXED */
    /* Preconditioner of the mixed-precision CG_nomass solve (not a reference parameter: the reference and the
     * FP64 path always precondition with the Jacobi diagonal). 0: the default (FFEA_GPU_CG_POLY_DEFAULT);
     * -1: Jacobi alone; 2, 4, 6 or 8: a Chebyshev polynomial of that degree in D^-1 V times the Jacobi scaling,
     * which needs fewer iterations and the same stopping test (|r|^2/|f|^2 < epsilon2). The polynomial applies when
     * the single-reduction kernel runs (the blob's rows fit in the GPU's shared memory); the blob's first solve
     * uses Jacobi and estimates the largest eigenvalue of D^-1 V for the later ones. */
    int cg_poly;
    /* Shared-memory copy of the matrix in the mixed-precision single-reduction CG_nomass kernel (not a reference
     * parameter): each block keeps the first 3x3 blocks of its owned rows on chip for the whole solve.
     * 0: as many as fit (the default); n > 0: at most n per row; -1: none. The results do not depend on it
     * (only where the matrix is read from), so it exists for measurements of the cache's effect. */
    int cg_smem_blocks;
} ffea_gpu_params;
#define FFEA_GPU_CG_POLY_DEFAULT 6
#define FFEA_GPU_CG_POLY_MAX 8  /* the highest Chebyshev degree cg_poly accepts (even degrees only) */

/* SimulationParams::SimulationParams() defaults for the hot-path fields
 * (src/SimulationParams.cpp:26-60); solver CG_nomass, precision FP64. */
int ffea_gpu_params_default(ffea_gpu_params *p);

/* SimulationParams::assign for one `<key = value>` of a .ffea <param> block
 * (src/SimulationParams.cpp:245-560): SI -> meso conversion for dt, kT,
 * stokes_visc; epsilon is squared; calc_stokes also accepts do_stokes.
 * Keys outside the hot path return FFEA_GPU_EINPUT. */
int ffea_gpu_params_assign(ffea_gpu_params *p, const char *key, const char *value);

/* Blob::load_material_params per-element conversion (src/Blob.cpp:2275-2283):
 * mat6 = n x {density, shear_visc, bulk_visc, shear_mod, bulk_mod, dielectric} (SI)
 * -> rho, A, B, G, E in meso units, including the reference's second-viscosity
 * expression B = bulk_visc/(P t) - (2/3) shear_visc. */
int ffea_gpu_material_from_si(int n, const double *mat6, double *rho, double *A, double *B, double *G, double *E);

/* a blob's structure in the units the reference holds after Blob::init loads it */
typedef struct ffea_gpu_mesh {
    int num_nodes;              /* all nodes, vertices and edge midpoints */
    int num_elements;
    int num_pinned;
    const double *pos;          /* 3 * num_nodes, meso */
    const int *tets;            /* 10 * num_elements, node indices (4 vertices then 6 midpoints) */
    const double *rho, *A, *B, *G, *E; /* num_elements each, meso */
    const double *stokes_radius;       /* num_nodes, meso (may be NULL when calc_stokes == 0) */
    const int *pinned;          /* num_pinned node indices */
} ffea_gpu_mesh;

typedef struct ffea_gpu_blob ffea_gpu_blob;

/* Blob::config + Blob::init (src/Blob.cpp:108-365) + Solver::init: rest state
 * (calc_rest_state_info :3080-3143), node-element connectivity (:3284-3314),
 * fixed sparsity pattern (NoMassCGSolver::init, src/NoMassCGSolver.cpp:56-153;
 * ConjugateGradientSolver::init; MassLumpedSolver::init) and device upload. */
int ffea_gpu_blob_create(const ffea_gpu_mesh *mesh, const ffea_gpu_params *params, ffea_gpu_blob **out);

/* Same from the reference's structure files (.node/.top/.mat/.stokes/.pin; pin may be NULL),
 * with `scale` the .ffea scale in metres per file unit (src/World.cpp:2632). */
int ffea_gpu_blob_load(const char *node_file, const char *top_file, const char *mat_file, const char *stokes_file,
                       const char *pin_file, double scale, const ffea_gpu_params *params, ffea_gpu_blob **out);

void ffea_gpu_blob_destroy(ffea_gpu_blob *blob);

/* The state of the blob's RngStream (RngStream::SetSeed/GetState semantics:
 * 6 integers, the first three < 4294967087, the last three < 4294944443).
 * Draws are consumed in the reference's single-thread order: 7 per element in
 * element order (tetra_element_linear::add_fluctuating_stress), then 3 per
 * node in node order when Stokes noise is on (src/Blob.cpp:3172-3224). A
 * reference run with OMP_NUM_THREADS=1 seeded with the package seed s uses
 * exactly the stream whose state is s. */
int ffea_gpu_blob_set_rng_state(ffea_gpu_blob *blob, const uint32_t state[6]);
int ffea_gpu_blob_get_rng_state(ffea_gpu_blob *blob, uint32_t state[6]);

/* nsteps x { Blob::zero_force; set_forces_to_zero; update_internal_forces;
 * update_positions } (the per-blob slice of World::run, src/World.cpp:1788-2059).
 * Stops at the first failing step; *steps_done (may be NULL) gets the number
 * of completed steps. */
int ffea_gpu_blob_step(ffea_gpu_blob *blob, int nsteps, int *steps_done);

/* Phases of one step, in launch order (for ffea_gpu_blob_step_timed). */
#define FFEA_GPU_NUM_PHASES 5 /* 0 element stress/forces, 1 matrix assembly, 2 force gather, 3 CG solve, 4 Euler */

/* ffea_gpu_blob_step, with every step timed by CUDA events on the blob's stream.
 * Before each step, flush_bytes of scratch device memory are written (outside the
 * timed window) so that each step starts with a cold L2; 0 disables the flush.
 * *step_ms gets the summed device time of the steps; phase_ms (may be NULL) gets
 * FFEA_GPU_NUM_PHASES per-phase sums (events between the kernels of each step). With
 * phase_ms NULL the steps run without those inner events (each step is timed by
 * events around its graph launch alone), as ffea_gpu_blob_step runs them. */
int ffea_gpu_blob_step_timed(ffea_gpu_blob *blob, int nsteps, long long flush_bytes, int *steps_done,
                             double *step_ms, double *phase_ms);

/* Host state in the reference's node order, all nodes (midpoints rebuilt). Any pointer may be NULL. */
int ffea_gpu_blob_get_state(ffea_gpu_blob *blob, double *pos, double *vel, double *force);
/* Overwrite positions (3 * num_nodes, meso; midpoint entries are ignored) and/or velocities. */
int ffea_gpu_blob_set_state(ffea_gpu_blob *blob, const double *pos, const double *vel);

/* Blob::make_measurements energies (src/Blob.cpp:1066-1125), meso units. */
int ffea_gpu_blob_measure(ffea_gpu_blob *blob, double *strain_energy, double *kinetic_energy);

/* Constant forces of the reference's ctforces file for blob `blob_index` (Blob::load_ctforces,
 * src/Blob.cpp:2478-2805; applied as Blob::apply_ctforces, :1676-1743): linear forces on nodes (added
 * before the element forces), rotational forces about an axis through a point ("pf", "pt": evaluated at
 * the nodes' current positions every step, after the linear ones), and linear surface forces spread over
 * sets of faces of `surface_file` (the blob's .surf; may be NULL without surface forces) in proportion to
 * their current areas (added after the element forces, face by face). Rotational forces about an axis
 * between two nodes return FFEA_GPU_EINPUT: the reference reads them but never applies them. Replaces
 * any constant forces loaded before. */
int ffea_gpu_blob_load_ctforces(ffea_gpu_blob *blob, const char *ctforces_file, const char *surface_file,
                                int blob_index);

/* All of Blob::make_measurements (src/Blob.cpp:1066-1202), reduced on the device in FP64:
 * out[0] strain energy, out[1] kinetic energy (0 for CG_nomass), out[2..4] centroid of all nodes,
 * out[5] RMSD of all nodes from the reference positions (meso units). The reference positions are
 * the positions at creation until ffea_gpu_blob_set_rmsd_reference (Blob::set_pos_0) replaces
 * them with the current ones. */
int ffea_gpu_blob_measurements(ffea_gpu_blob *blob, double out[6]);
int ffea_gpu_blob_set_rmsd_reference(ffea_gpu_blob *blob);

/* CG iterations of the last step and in total (0 for masslumped). */
int ffea_gpu_blob_cg_iterations(ffea_gpu_blob *blob, int *last, long long *total);

/* Relative squared residual |r|^2/|f|^2 after each CG iteration of the last solve (the quantity
 * NoMassCGSolver::solve tests against epsilon2); *count gets the number written (<= max_entries). */
int ffea_gpu_blob_cg_history(ffea_gpu_blob *blob, double *res2, int max_entries, int *count);

/* Where the last CG solve spent its time, as seen by one thread block (device timer, ns, summed
 * over iterations): [0] set-up, [1] SpMV, [2] block reduction after the SpMV, [3] grid barrier
 * after the SpMV, [4] cross-block sums and step length, [5] solution/residual update, [6] its block
 * reduction, [7] its grid barrier, [8] its cross-block sums, [9] direction update and its barrier
 * (FP64 path only). n_phases is 10. */
#define FFEA_GPU_CG_PHASES 10
int ffea_gpu_blob_cg_profile(ffea_gpu_blob *blob, double *phase_ns, int n_phases);

/* The preconditioner the blob's next CG solve uses: *degree is the Chebyshev polynomial's degree (0: Jacobi,
 * always so on the FP64 path, before the first solve, and when the trial solve found Jacobi cheaper) and
 * *lambda_max the estimate of the largest eigenvalue of D^-1 V it is built on (0 without one). Each CG
 * iteration then applies the matrix 1 + degree times. */
int ffea_gpu_blob_cg_preconditioner(ffea_gpu_blob *blob, int *degree, double *lambda_max);

/* Name of the persistent CG kernel the blob's steps launch, fixed at creation by the blob's size and
 * precision alone (static string; "none" for masslumped, which solves no system):
 *   FP64: "cg_own_kernel" (each block keeps its rows on chip) or "cg_kernel" (grid-strided, larger blobs);
 *   mixed: "cg_mixed_sr_kernel" (CG_nomass, one reduction per iteration, FP32 matrix up to 64 MB so that it
 *   stays in L2), "cg_mixed_own_kernel" (two reductions, rows on chip) or "cg_mixed_kernel" (grid-strided). */
const char *ffea_gpu_blob_cg_kernel(ffea_gpu_blob *blob);

/* Nodes of the reference numbering (vertices and midpoints) and elements of the blob. */
int ffea_gpu_blob_counts(ffea_gpu_blob *blob, int *num_nodes, int *num_elements);

/* Problem sizes: vertex nodes, elements, matrix 3x3 blocks. */
int ffea_gpu_blob_sizes(ffea_gpu_blob *blob, int *num_linear_nodes, int *num_elements, long long *num_blocks);

/* NoMass viscosity matrix in the reference's scalar CSR over all 3*num_nodes
 * rows (SparsityPattern::create_sparse_matrix, src/SparsityPattern.cpp:69-110):
 * key has 3*num_nodes+1 entries; col and val have *nnz entries. Call once
 * with col == NULL to get *nnz. val holds the values of the last assembly;
 * nsrc (may be NULL) the number of summed sources per entry. */
int ffea_gpu_blob_get_pattern(ffea_gpu_blob *blob, int *key, int *col, double *val, int *nsrc, long long *nnz);

/* Node -> (element*10 + slot) force-contribution lists in the reference's
 * order (Blob::calculate_node_element_connectivity, src/Blob.cpp:3284-3314);
 * ptr has num_nodes+1 entries. Call with elem_slot == NULL to get *count. */
int ffea_gpu_blob_get_connectivity(ffea_gpu_blob *blob, int *ptr, int *elem_slot, long long *count);

/* Per-element outputs of the last update_internal_forces: node forces of the
 * four vertices (12 per element: node-major xyz, as tetra_element_linear::node_force[0..3]),
 * volume, and the 12x12 viscosity matrix (144 per element, may be NULL). */
int ffea_gpu_blob_get_elements(ffea_gpu_blob *blob, double *node_force12, double *vol, double *visc144);

/* The assembled force vector of the last step (solver input, 3 * num_nodes, midpoints zero). */
int ffea_gpu_blob_get_rhs(ffea_gpu_blob *blob, double *rhs);

/* Allocation-free solve. No counterpart in the reference (the nearest is
 * Solver::solve, include/Solver.h:31-52, as NoMassCGSolver::solve,
 * src/NoMassCGSolver.cpp:156-188, and ConjugateGradientSolver::solve,
 * src/ConjugateGradientSolver.cpp:193-217).
 *
 * Solves M x = rhs with the blob's current matrix (CG_nomass: the viscosity
 * matrix assembled by the last ffea_gpu_blob_step; CG: the constant mass
 * matrix) by the grid-strided persistent Jacobi-PCG kernel, from x = 0, with
 * the blob's epsilon and max_iterations_cg. A step may run another CG kernel
 * (one whose blocks keep their rows on chip) that sums in another order, so
 * the two solutions agree to rounding and their iteration counts may differ
 * by one. rhs and x hold 3 * num_nodes doubles
 * in the layout of ffea_gpu_blob_get_rhs and may be the same array; midpoint
 * rows are identity rows (x = rhs there). *iterations (may be NULL) gets the
 * CG iterations used. Returns FFEA_GPU_ECGMAXIT / FFEA_GPU_ETIMEOUT like a step.
 *
 * It allocates no memory, on the device or through any library: every work
 * array comes from one static device array of this library, sized for
 * FFEA_GPU_SOLVE_STATIC_MAX_NODES vertex nodes (4.99 MB). Blobs with more
 * vertex nodes, mixed-precision blobs and mass-lumped blobs are rejected with
 * FFEA_GPU_EINPUT and a message in ffea_gpu_last_error. The array is placed
 * on a device (cudaGetSymbolAddress, which loads the library's module there)
 * by the creation of the first blob that this call accepts, so the first call
 * allocates nothing either; a caller who fills the GPU's memory should create
 * its blobs first. The call makes the blob's device current and restores the
 * caller's on return. The array is shared by all calls on a device, so two
 * calls whose kernels overlapped would corrupt each other: each call holds a
 * process-wide lock and waits for its kernels to finish (on success and on
 * error) before it returns, so calls from several host threads run one after
 * another. */
#define FFEA_GPU_SOLVE_STATIC_MAX_NODES 32768
int ffea_gpu_blob_solve_static(ffea_gpu_blob *blob, const double *rhs, double *x, int *iterations);

/* ---------------------------------------------------------------------------
 * Adjoint of a window of CG_nomass steps (the reference has no derivative code;
 * this differentiates the step of ffea_gpu_blob_step).
 *
 * create: reserves checkpoint storage on `blob` for a window of window_steps steps
 *   with a checkpoint (positions, stream state, element determinants) every
 *   checkpoint_every steps. One adjoint per blob. Destroying the blob first
 *   leaves the adjoint inert (its calls return FFEA_GPU_EINPUT); destroy it after.
 * forward: runs the window from the blob's current state (as ffea_gpu_blob_step),
 *   storing the checkpoints; the blob ends at the window's last state.
 * backward: given dL/dx_final (3 * num_nodes, reference node order, midpoints
 *   allowed), recomputes each segment from its checkpoint with the same noise
 *   draws and runs the reverse sweep: one adjoint CG solve with the step's
 *   viscosity matrix per step, plus the hand-written element derivative. Writes
 *   dL/dG, dL/dE, dL/dA, dL/dB per element (meso units, the parameters of
 *   ffea_gpu_mesh; any may be NULL) and dL/dx_initial (3 * num_nodes, may be
 *   NULL). The blob is left at the window's last state.
 * ------------------------------------------------------------------------- */
typedef struct ffea_gpu_adjoint ffea_gpu_adjoint;
int ffea_gpu_adjoint_create(ffea_gpu_blob *blob, int window_steps, int checkpoint_every, ffea_gpu_adjoint **out);
int ffea_gpu_adjoint_forward(ffea_gpu_adjoint *adj, int *steps_done);
int ffea_gpu_adjoint_backward(ffea_gpu_adjoint *adj, const double *dl_dx_final, double *dl_dG, double *dl_dE,
                              double *dl_dA, double *dl_dB, double *dl_dx_initial);
void ffea_gpu_adjoint_destroy(ffea_gpu_adjoint *adj);

/* ---------------------------------------------------------------------------
 * Replica batch: many independent blobs of uneven size advanced together.
 *
 * The reference advances the blobs of a World one after another with the same
 * per-blob slice of World::run (src/World.cpp:1788-2059); a batch runs that
 * slice for every blob at once: one CUDA graph per step, one persistent
 * cooperative CG launch in which each blob's CTA group iterates until its own
 * blob has converged. Mixed precision and the CG_nomass solver only. Blob b's
 * noise comes from substream b of the stream whose state is the package seed
 * 12345 x 6 (RngStream::ResetNextSubstream applied b times), drawn in the
 * reference's single-thread order within the blob: 7 per element, then (Stokes
 * drag with noise) 3 per node of the blob's own numbering.
 * ------------------------------------------------------------------------- */
typedef struct ffea_gpu_batch ffea_gpu_batch;
#define FFEA_GPU_BATCH_MAX_BLOBS 2048

/* meshes[b] as for ffea_gpu_blob_create; params shared by every blob. Every blob needs a CTA of the CG launch
 * resident at once, so num_blobs is also bounded by the GPU's resident CTAs of 128 threads (1,216 on a GB300);
 * above either bound FFEA_GPU_EINPUT. */
int ffea_gpu_batch_create(const ffea_gpu_mesh *meshes, int num_blobs, const ffea_gpu_params *params,
                          ffea_gpu_batch **out);
void ffea_gpu_batch_destroy(ffea_gpu_batch *batch);

/* Totals over the batch: blobs, vertex nodes, elements, nonzero 3x3 matrix blocks. */
int ffea_gpu_batch_sizes(ffea_gpu_batch *batch, int *num_blobs, int *vertex_nodes, int *elements, long long *blocks);
/* One blob: all nodes (the length of its state arrays / 3), vertex nodes, elements. */
int ffea_gpu_batch_blob_sizes(ffea_gpu_batch *batch, int blob, int *num_nodes, int *vertex_nodes, int *elements);

/* nsteps steps of every blob; stops at the first failing step (*steps_done gets the completed steps). */
int ffea_gpu_batch_step(ffea_gpu_batch *batch, int nsteps, int *steps_done);
/* Same, each step timed by CUDA events around its graph launch, with flush_bytes of scratch written
 * before every step outside the timed window; *step_ms = summed device time. cg_ms (may be NULL): the
 * summed time of the steps' CG launches (events recorded around it inside the step). */
int ffea_gpu_batch_step_timed(ffea_gpu_batch *batch, int nsteps, long long flush_bytes, int *steps_done,
                              double *step_ms, double *cg_ms);

/* State of one blob in its own node order (as ffea_gpu_blob_get_state / set_state). */
int ffea_gpu_batch_get_state(ffea_gpu_batch *batch, int blob, double *pos, double *vel);
int ffea_gpu_batch_set_state(ffea_gpu_batch *batch, int blob, const double *pos, const double *vel);
/* Every blob's state at once: the blobs' arrays back to back in blob order (sum of the blobs' node
 * counts x 3 doubles each), as num_blobs calls of ffea_gpu_batch_get_state / set_state, with one host <->
 * device transfer. */
int ffea_gpu_batch_get_states(ffea_gpu_batch *batch, double *pos, double *vel);
int ffea_gpu_batch_set_states(ffea_gpu_batch *batch, const double *pos, const double *vel);
int ffea_gpu_batch_set_rng_state(ffea_gpu_batch *batch, int blob, const uint32_t state[6]);
int ffea_gpu_batch_get_rng_state(ffea_gpu_batch *batch, int blob, uint32_t state[6]);

/* Each blob's strain energy (the StrainEnergy of Blob::make_measurements, src/Blob.cpp:1066-1125; meso units)
 * at the current positions, in FP64: out[num_blobs]. */
int ffea_gpu_batch_strain_energies(ffea_gpu_batch *batch, double *out);

/* Constant forces of blob `blob` of the batch, read as ffea_gpu_blob_load_ctforces reads them (the
 * ctforces file's entries for `blob_index`, faces of `surface_file`); each call replaces that blob's
 * forces only. */
int ffea_gpu_batch_load_ctforces(ffea_gpu_batch *batch, int blob, const char *ctforces_file,
                                 const char *surface_file, int blob_index);

/* CG iterations of each blob's last solve (num_blobs entries, may be NULL) and the total since creation. */
int ffea_gpu_batch_cg_iterations(ffea_gpu_batch *batch, int *last_per_blob, long long *total);

/* Launch configuration of the batch CG: CTA size, threads per matrix row, CTAs in the grid. */
int ffea_gpu_batch_config(ffea_gpu_batch *batch, int *cg_threads, int *threads_per_row, int *ctas);
int ffea_gpu_batch_set_config(ffea_gpu_batch *batch, int cg_threads, int threads_per_row);

/* Launch shapes of the force phase: elements per thread block of the element kernel (64, 128, 256; the
 * block's vertices are staged in shared memory and its forces summed per vertex there), threads per
 * block of the assembly (64, 128, 256) and its slot split (0: three threads per matrix slot while they
 * fit on the GPU at once, 1: three, 2: one), threads per block of the node-force gather (64, 128, 256).
 * Any shape gives the same trajectory to FP32 rounding (the block sums change grouping). */
int ffea_gpu_batch_shapes(ffea_gpu_batch *batch, int *element_threads, int *assembly_threads, int *assembly_split,
                          int *gather_threads);
int ffea_gpu_batch_set_shapes(ffea_gpu_batch *batch, int element_threads, int assembly_threads,
                              int assembly_split, int gather_threads);

/* Autotuner. First the force phase (node preparation, elements, assembly, node forces), timed over
 * `solves` launches per shape and searched one shape at a time: elements per block, then the
 * assembly's threads and split, then the gather's threads. Then `solves` CG solves of the current
 * forces for every CTA size (128..1024) and threads per row (1, 2, 4, 8). Keeps the fastest of each;
 * positions, velocities and RNG states are not changed. *best_ms (may be NULL) gets the best mean solve
 * time. */
int ffea_gpu_batch_tune(ffea_gpu_batch *batch, int solves, double *best_ms);

/* ---------------------------------------------------------------------------
 * .ffea script front-end: a World with the blob-step path only
 * (World::init / World::run, src/World.cpp:54-620, 1747-2059).
 *
 * load: reads the script's <param> and <system> blocks (one conformation per
 *   blob), builds each blob from its structure files, applies centroid /
 *   rotation / velocity and the move into the simulation box, sets the RMSD
 *   reference, seeds the stream from rng_seed (or, with restart = 1, from
 *   checkpoint_in and the trajectory's last complete frame), loads each blob's
 *   constant forces (calc_ctforces = 1) and opens the trajectory and
 *   measurement files. Features outside the path (calc_ssint, calc_steric,
 *   calc_es, kinetics, springs, preComp, rods, several conformations, STATIC
 *   blobs) are refused with FFEA_GPU_EINPUT.
 * run: steps step_initial .. num_steps; every `check` steps the stream state
 *   goes to checkpoint_out before the forces, then the positions to the
 *   trajectory (.ftj) and the measurements (.fm), as the reference writes them.
 * ------------------------------------------------------------------------- */
typedef struct ffea_gpu_world ffea_gpu_world;
int ffea_gpu_world_load(const char *ffea_script, int precision, ffea_gpu_world **out);
int ffea_gpu_world_run(ffea_gpu_world *world, long long *last_step);
int ffea_gpu_world_num_blobs(ffea_gpu_world *world);
ffea_gpu_blob *ffea_gpu_world_blob(ffea_gpu_world *world, int index);
void ffea_gpu_world_destroy(ffea_gpu_world *world);

/* Last CUDA error text for FFEA_GPU_ECUDA (static storage). */
const char *ffea_gpu_last_error(void);

/* Kernel launches issued by this library since load (for benchmarking claims). */
long long ffea_gpu_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
