/*
 * ffea_oracle.h -- CPU restatement of FFEA's per-timestep blob update.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle that the CUDA path is checked
 * against; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it. The product library never links or calls it.
 *
 * It restates, in plain C with OpenMP, the algorithm of the reference
 * (RSE-Sheffield/ffea_ci_demo, FFEA 2.7.2) for the hot path:
 *   Blob::update_internal_forces      src/Blob.cpp:400-491
 *   Blob::aggregate_forces_and_solve  src/Blob.cpp:3147-3244
 *   Blob::euler_integrate             src/Blob.cpp:3249-3279
 *   NoMassCGSolver                    src/NoMassCGSolver.cpp:56-281
 *   ConjugateGradientSolver           src/ConjugateGradientSolver.cpp:51-334
 *   MassLumpedSolver                  src/MassLumpedSolver.cpp:27-72
 *   RngStream (MRG32k3a)              src/RngStream.cpp
 * The data layout mirrors the reference (10-node elements, every node kept,
 * scalar CSR of {int column, double value} entries whose values are re-summed
 * each step from per-element source pointers), so that timing it is timing
 * the reference's algorithm on the same data structures.
 */
#ifndef FFEA_ORACLE_H
#define FFEA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- MRG32k3a stream (RngStream restated) ---- */
typedef struct orc_rng {
    uint32_t Cg[6], Bg[6], Ig[6];
    int anti, inc_prec;
} orc_rng;

void orc_rng_set_package_seed(const uint32_t seed[6]);      /* RngStream::SetPackageSeed */
int orc_rng_check_seed(const uint32_t seed[6]);              /* 0 ok, -1 invalid */
void orc_rng_create(orc_rng *g);                             /* RngStream::RngStream() */
void orc_rng_reset_start_stream(orc_rng *g);
void orc_rng_reset_start_substream(orc_rng *g);
void orc_rng_reset_next_substream(orc_rng *g);
void orc_rng_advance_state(orc_rng *g, int32_t e, int32_t c);
void orc_rng_set_antithetic(orc_rng *g, int a);
void orc_rng_increased_precis(orc_rng *g, int p);
double orc_rng_rand_u01(orc_rng *g);
int orc_rng_rand_int(orc_rng *g, int lo, int hi);
void orc_rng_get_state(const orc_rng *g, uint32_t out[6]);
void orc_rng_set_state(orc_rng *g, const uint32_t s[6]);     /* Cg = Bg = Ig = s */
/* World::init seeding from an integer rng_seed (src/World.cpp:270-288) */
void orc_seed_from_rng_seed(int rng_seed, uint32_t out[6]);

/* ---- blob ---- */
enum { ORC_NOMASS_CG = 0, ORC_CG = 1, ORC_MASSLUMPED = 2 };
enum { ORC_OK = 0, ORC_EINVERTED = 1, ORC_ECGMAXIT = 2, ORC_EINPUT = 3, ORC_ENOMEM = 4 };

typedef struct orc_params {
    /* SI values as written in a .ffea <param> block */
    double dt, kT, epsilon, stokes_visc;
    int max_iterations_cg, calc_noise, calc_stokes;
} orc_params;

typedef struct orc_blob orc_blob;

/*
 * pos: 3*n_nodes file-unit coordinates, multiplied by scale/mesoDimensions::length
 * tets: 10*n_elem node indices; mat6: 6*n_elem SI (rho, eta_s, eta_b, G, K, eps_r)
 * stokes_radius: n_nodes file units (multiplied like positions)
 * n_threads: OpenMP threads (and RngStreams, one per thread as in World::init)
 */
orc_blob *orc_blob_create(int n_nodes, const double *pos, double scale_m, int n_elem, const int *tets,
                          const double *mat6, const double *stokes_radius, int n_pinned, const int *pinned,
                          const orc_params *p, int solver, int n_threads, int *status);
void orc_blob_destroy(orc_blob *b);
/* one World::run step slice for this blob; returns ORC_* */
int orc_blob_step(orc_blob *b, int nsteps);
/* pieces of a step, for per-kernel parity */
int orc_blob_update_internal_forces(orc_blob *b);
int orc_blob_update_positions(orc_blob *b);
void orc_blob_zero_forces(orc_blob *b);

int orc_blob_n_nodes(const orc_blob *b);
int orc_blob_n_elem(const orc_blob *b);
void orc_blob_get_pos(const orc_blob *b, double *out);       /* 3*n_nodes, meso */
void orc_blob_set_pos(orc_blob *b, const double *in);        /* 3*n_nodes, meso; then re-linearise */
void orc_blob_get_vel(const orc_blob *b, double *out);
void orc_blob_get_force(const orc_blob *b, double *out);     /* last solver output (v or a) */
void orc_blob_get_rhs(const orc_blob *b, double *out);       /* last assembled force (solver input) */
/* per element: node_force[4][3] (12), dpsi (12), vol, vol_0, viscosity matrix (144), stress mag */
void orc_blob_get_elem(const orc_blob *b, double *node_force12, double *dpsi12, double *vol, double *vol0,
                       double *visc144, double *stress_mag);
/* rest state: J_inv_0 (9 per element) and converted material (rho,A,B,G,E per element) */
void orc_blob_get_rest(const orc_blob *b, double *jinv9, double *mat5);
double orc_blob_param(const orc_blob *b, const char *name);
/* NoMass viscosity CSR (after the last build) */
int orc_blob_nnz(const orc_blob *b);
void orc_blob_get_csr(const orc_blob *b, int *key, int *col, double *val, int *nsrc);
/* node -> (element*10+slot) contribution lists, reference order */
int orc_blob_n_contrib(const orc_blob *b);
void orc_blob_get_contrib(const orc_blob *b, int *ptr, int *elem_slot);
/* consistent-mass CSR (solver CG) */
int orc_blob_mass_nnz(const orc_blob *b);
void orc_blob_get_mass_csr(const orc_blob *b, int *key, int *col, double *val);
void orc_blob_get_inv_mass(const orc_blob *b, double *out);  /* masslumped inv_M */
int orc_blob_last_cg_iters(const orc_blob *b);
long long orc_blob_total_cg_iters(const orc_blob *b);
void orc_blob_get_rng_state(const orc_blob *b, int stream, uint32_t out[6]);
void orc_blob_set_rng_state(orc_blob *b, int stream, const uint32_t s[6]);
/* Blob::make_measurements energies: strain energy and kinetic energy (meso) */
void orc_blob_measure(const orc_blob *b, double *strain_energy, double *kinetic_energy);
/*
 * Constant forces of this blob (Blob::load_ctforces, src/Blob.cpp:2478-2805), as read from the file:
 *   linear forces (CTF 1): n_lin entries in file order, node lin_node[i], force magnitude and direction
 *     lin_fd[4i..4i+3] = (F [N], dx, dy, dz), "all" already expanded to one entry per node;
 *   linear surface forces (CTF 3): n_sets sets, set s holding set_size[s] faces (concatenated in set_faces)
 *     and set_fd[4s..4s+3] = (F [N], dx, dy, dz);
 *   the surface: n_faces faces of three nodes each (face_nodes), as in the .surf file.
 * Returns ORC_OK, or ORC_EINPUT for an index out of range or a zero direction.
 */
int orc_blob_set_ctforces(orc_blob *b, int n_lin, const int *lin_node, const double *lin_fd, int n_sets,
                          const int *set_size, const int *set_faces, const double *set_fd, int n_faces,
                          const int *face_nodes);
/*
 * Rotational constant forces (CTF 2) of this blob, after orc_blob_set_ctforces, in file order ("all" expanded):
 * node rot_node[i], type rot_torque[i] (0: "pf", 1: "pt"), rot_fpd[7i..7i+6] = (F [N], px, py, pz [m], dx, dy, dz).
 * Returns ORC_OK, or ORC_EINPUT for a node out of range or a zero axis.
 */
int orc_blob_set_rot_ctforces(orc_blob *b, int n_rot, const int *rot_node, const int *rot_torque,
                              const double *rot_fpd);

#ifdef __cplusplus
}
#endif
#endif
