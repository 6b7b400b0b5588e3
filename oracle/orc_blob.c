/*
 * orc_blob.c -- CPU restatement of one FFEA blob time step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle; see ffea_oracle.h). Compiled with
 * -ffp-contract=off so that every floating-point expression is evaluated in
 * the reference's source order with IEEE rounding and no fused multiply-add.
 *
 * Every function below names the reference code it restates.
 */
#include "ffea_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* mesoDimensions, include/dimensions.h:30-41 */
#define MESO_LENGTH 1.7e-10
#define MESO_ENERGY 4.141945559999999e-21
#define MESO_MASS 1.994307387553024e-26
#define MESO_VOLUME 4.913e-30
#define MESO_TIME 3.7302915560886126e-13
#define MESO_PRESSURE 8.4305832688784826e8
#define MESO_FORCE 2.4364705882352941e-11
#define FFEA_PI 3.141592653589793238462643383279502884197169399375105820974944592307816406286208998628034825342117067982148

typedef struct { int col; double val; } orc_entry; /* sparse_entry, include/SparseMatrixTypes.h:31-35 */

struct orc_blob {
    int n, T, solver, nthreads;
    double dt, kT, eps2, stokes_visc;
    int imax, calc_noise, calc_stokes;
    /* nodes (mesh_node) */
    double *pos, *vel, *force, *rhs, *stokes_radius, *stokes_drag;
    int *is_pinned, *pinned, npinned;
    /* elements (tetra_element_linear) */
    int *tet;
    double *rho, *A, *B, *G, *E, *vol0, *vol, *last_det, *jinv0, *dpsi, *visc, *node_force, *F, *stress_mag;
    /* connectivity (Blob::calculate_node_element_connectivity) */
    int *cptr;
    double **contrib;
    int *contrib_es;
    /* NoMassCGSolver */
    int rows, nnz;
    int *key;
    orc_entry *entry;
    int *sptr;
    double **src;
    double **diag;
    double one;
    double *precond, *r, *p, *z, *q, *f, *work_in, *work_out;
    /* ConjugateGradientSolver (scalar mass CSR over nodes) */
    int mnnz;
    int *mkey;
    orc_entry *mentry;
    double *d, *s;
    /* MassLumpedSolver */
    double *inv_m;
    /* RNG, one stream per thread (World::init, src/World.cpp:259-300) */
    orc_rng *rng;
    int last_iters;
    long long total_iters;
    /* constant forces (Blob::load_ctforces, src/Blob.cpp:2478-2805): ctf_l_nodes / ctf_l_forces,
     * ctf_sl_surfsize / ctf_sl_faces / ctf_sl_forces, and the surface faces with their Face::force */
    int n_lctf, n_sets, n_faces;
    int *lctf_node, *set_size, *set_faces, *face_nodes;
    double *lctf_f, *set_f, *face_f, *face_area;
    /* rotational constant forces: ctf_r_nodes, ctf_r_forces, ctf_r_axis (point, direction), ctf_r_type */
    int n_rctf;
    int *rctf_node, *rctf_torque;
    double *rctf_f, *rctf_axis;
};

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz ? sz : 1); }

/* ---------------------------------------------------------------------------
 * element kernel pieces -- src/tetra_element_linear.cpp
 * ------------------------------------------------------------------------- */

/* calculate_jacobian, :191-203 */
static void elem_jacobian(const orc_blob *b, int e, double J[3][3]) {
    const int *t = b->tet + 10 * (size_t)e;
    const double *x0 = b->pos + 3 * (size_t)t[0];
    for (int r = 0; r < 3; ++r) {
        const double *xr = b->pos + 3 * (size_t)t[r + 1];
        J[r][0] = xr[0] - x0[0];
        J[r][1] = xr[1] - x0[1];
        J[r][2] = xr[2] - x0[2];
    }
}

/* calc_shape_function_derivatives_and_volume, :222-292; returns 1 if inverted */
static int elem_dpsi_vol(orc_blob *b, int e, double J[3][3]) {
    double *dpsi = b->dpsi + 12 * (size_t)e;
    dpsi[1] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    dpsi[2] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    dpsi[3] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    dpsi[5] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
    dpsi[6] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
    dpsi[7] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
    dpsi[9] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
    dpsi[10] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
    dpsi[11] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
    double det = J[0][0] * dpsi[1] + J[1][0] * dpsi[2] + J[2][0] * dpsi[3];
    if (b->last_det[e] * det < 0) return 1;
    b->last_det[e] = det;
    b->vol[e] = (1.0 / 6.0) * fabs(det);
    det = 1.0 / det;
    dpsi[1] *= det; dpsi[2] *= det; dpsi[3] *= det;
    dpsi[5] *= det; dpsi[6] *= det; dpsi[7] *= det;
    dpsi[9] *= det; dpsi[10] *= det; dpsi[11] *= det;
    dpsi[0] = -(dpsi[1] + dpsi[2] + dpsi[3]);
    dpsi[4] = -(dpsi[5] + dpsi[6] + dpsi[7]);
    dpsi[8] = -(dpsi[9] + dpsi[10] + dpsi[11]);
    return 0;
}

/* create_viscosity_matrix, :298-327, with BULK_VISCOUS_SUBMATRIX_DIAG/OFFDIAG
 * (include/tetra_element_linear.h:56-117), calc_del2_matrix (:585-605) and
 * add_diffusion_matrix (:607-622). */
static void elem_viscosity(orc_blob *b, int e) {
    const double *dpsi = b->dpsi + 12 * (size_t)e;
    double (*V)[12] = (double (*)[12])(b->visc + 144 * (size_t)e);
    const double A = b->A[e], B = b->B[e];
    for (int I = 0; I < 12; I += 4) {          /* diagonal 4x4 blocks, upper triangle */
        for (int a = 0; a < 4; ++a)
            for (int c = a; c < 4; ++c) V[I + a][I + c] = dpsi[I + a] * dpsi[I + c] * (A + B);
    }
    const int off[3][2] = {{0, 4}, {0, 8}, {4, 8}};
    for (int o = 0; o < 3; ++o) {              /* off-diagonal 4x4 blocks */
        const int I = off[o][0], Jb = off[o][1];
        double K[4][4];
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 4; ++c) K[a][c] = dpsi[I + a] * dpsi[Jb + c];
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 4; ++c)
                V[I + a][Jb + c] = (a == c) ? (B + A) * K[a][a] : B * K[a][c] + A * K[c][a];
    }
    double del2[4][4];
    for (int a = 0; a < 4; ++a)
        for (int c = a; c < 4; ++c)
            del2[a][c] = (dpsi[a] * dpsi[c] + dpsi[4 + a] * dpsi[4 + c] + dpsi[8 + a] * dpsi[8 + c]);
    for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 4; ++a)
            for (int c = a; c < 4; ++c) V[i * 4 + a][i * 4 + c] += del2[a][c] * A;
    const double vol = b->vol[e];
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j <= i; ++j) V[j][i] *= vol;
    for (int i = 1; i < 12; ++i)
        for (int j = 0; j < i; ++j) V[i][j] = V[j][i];
}

/* add_shear_elastic_stress :375-392 with mat3_mult_both_transposed,
 * mat3_mult_transpose, mat3_scale (src/mat_vec_fns.cpp:70-103) */
static void elem_shear_stress(orc_blob *b, int e, double J[3][3], double S[3][3]) {
    double *F = b->F + 9 * (size_t)e;
    const double *Ji = b->jinv0 + 9 * (size_t)e;
    for (int i = 0; i < 9; ++i) F[i] = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) F[3 * i + j] += J[k][i] * Ji[3 * j + k];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) S[i][j] += F[3 * i + k] * F[3 * j + k];
    const double s = (b->G[e] * b->vol0[e] / b->vol[e]);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S[i][j] *= s;
    S[0][0] -= b->G[e];
    S[1][1] -= b->G[e];
    S[2][2] -= b->G[e];
}

/* add_bulk_elastic_stress :397-403 */
static void elem_bulk_stress(const orc_blob *b, int e, double S[3][3]) {
    const double G = b->G[e], vol = b->vol[e], vol0 = b->vol0[e];
    const double c_2 = b->E[e] - G * 2.0 / 3.0;
    const double c = G * (1.0 - (vol0 / vol)) + 0.5 * c_2 * ((vol / vol0) - (vol0 / vol));
    S[0][0] += c;
    S[1][1] += c;
    S[2][2] += c;
}

/* RAND(-.5,.5), include/tetra_element_linear.h:119 */
static double rand_half(orc_rng *g) { return (-.5) + ((.5) - (-.5)) * orc_rng_rand_u01(g); }

/* add_fluctuating_stress :412-431 -- 7 draws in the order b, d0, d1, d2, o01, o02, o12 */
static void elem_fluct_stress(const orc_blob *b, int e, double S[3][3], orc_rng *g) {
    const double A = b->A[e], B = b->B[e];
    const double c = sqrt((24 * b->kT) / (b->vol[e] * b->dt));
    const double bf = sqrt(B) * rand_half(g);
    S[0][0] += c * (sqrt(2 * A) * rand_half(g) + bf);
    S[1][1] += c * (sqrt(2 * A) * rand_half(g) + bf);
    S[2][2] += c * (sqrt(2 * A) * rand_half(g) + bf);
    S[0][1] += c * sqrt(A) * rand_half(g);
    S[0][2] += c * sqrt(A) * rand_half(g);
    S[1][2] += c * sqrt(A) * rand_half(g);
    S[1][0] = S[0][1];
    S[2][0] = S[0][2];
    S[2][1] = S[1][2];
}

/* Blob::update_internal_forces, src/Blob.cpp:400-491 */
/* Face::get_area, src/Face.cpp:169-187: half the length of (n1 - n0) x (n2 - n0) */
static double face_get_area(const orc_blob *b, int f) {
    const double *p0 = b->pos + 3 * (size_t)b->face_nodes[3 * f], *p1 = b->pos + 3 * (size_t)b->face_nodes[3 * f + 1],
                 *p2 = b->pos + 3 * (size_t)b->face_nodes[3 * f + 2];
    double a[3], c[3], t[3];
    for (int i = 0; i < 3; ++i) {
        a[i] = p1[i] - p0[i];
        c[i] = p2[i] - p0[i];
    }
    t[0] = a[1] * c[2] - a[2] * c[1];
    t[1] = a[2] * c[0] - a[0] * c[2];
    t[2] = a[0] * c[1] - a[1] * c[0];
    /* magnitude, include/mat_vec_fns_II.h:326-333: an `omp simd` sum reduction, which GCC (-O2 -fopenmp,
     * two double lanes) evaluates as (t0^2 + t2^2) + t1^2; checked against the reference's header built so */
    const double r = (t[0] * t[0] + t[2] * t[2]) + t[1] * t[1];
    return .5 * sqrt(r);
}

/* arr3arr3VectorProduct, include/mat_vec_fns_II.h:369-373 */
static void cross3(const double *u, const double *v, double *w) {
    w[0] = u[1] * v[2] - v[1] * u[2];
    w[1] = -u[0] * v[2] + v[0] * u[2];
    w[2] = u[0] * v[1] - v[0] * u[1];
}

/* magnitude, include/mat_vec_fns_II.h:326-333, in the order GCC builds its two-lane `omp simd` sum */
static double magnitude3(const double *a) { return sqrt((a[0] * a[0] + a[2] * a[2]) + a[1] * a[1]); }

/* CTF 2 of Blob::apply_ctforces (src/Blob.cpp:1684-1720) for one entry at node position p0:
 * intersectingPointToLine (include/mat_vec_fns_II.h:755-777), r = p3 - p0, f = r x d, scaled by F or F/|r| */
static void rot_force(const double *axis, double F, int torque, const double *p0, double *f) {
    const double *p1 = axis, *d = axis + 3;
    double p0p1[3], v2[3], p3[3], r[3];
    for (int c = 0; c < 3; ++c) p0p1[c] = p0[c] - p1[c];
    cross3(p0p1, d, v2);
    if (magnitude3(v2) < 3.0 * 2.220446049250313080847e-16) {
        for (int c = 0; c < 3; ++c) p3[c] = p0[c];
    } else {
        double cp3p0[3], v1v2[3], cc;
        cross3(d, v2, cp3p0);
        cross3(d, cp3p0, v1v2);
        cc = p0p1[0] * (d[1] * v1v2[2] - d[2] * v1v2[1]); /* detByRows, :379-385 */
        cc += p0p1[1] * (d[2] * v1v2[0] - d[0] * v1v2[2]);
        cc += p0p1[2] * (d[0] * v1v2[1] - d[1] * v1v2[0]);
        cc /= (v1v2[0] * v1v2[0] + v1v2[1] * v1v2[1] + v1v2[2] * v1v2[2]);
        for (int c = 0; c < 3; ++c) p3[c] = p0[c] + cc * cp3p0[c];
    }
    for (int c = 0; c < 3; ++c) r[c] = p3[c] - p0[c];
    cross3(r, d, f);
    const double s = torque ? F / magnitude3(r) : F;
    for (int c = 0; c < 3; ++c) f[c] = s * f[c];
}

/* Blob::apply_ctforces, src/Blob.cpp:1676-1741 (CTF 1, CTF 2 about axes through a point, CTF 3) */
static void apply_ctforces(orc_blob *b) {
    for (int i = 0; i < b->n_lctf; ++i)
        for (int c = 0; c < 3; ++c) b->force[3 * (size_t)b->lctf_node[i] + c] += b->lctf_f[3 * i + c];
    for (int i = 0; i < b->n_rctf; ++i) {
        double f[3];
        const int n = b->rctf_node[i];
        rot_force(b->rctf_axis + 6 * i, b->rctf_f[i], b->rctf_torque[i], b->pos + 3 * (size_t)n, f);
        for (int c = 0; c < 3; ++c) b->force[3 * (size_t)n + c] += f[c];
    }
    int aux = 0;
    for (int s = 0; s < b->n_sets; ++s) {
        double total = 0;
        for (int j = 0; j < b->set_size[s]; ++j) {
            b->face_area[j] = face_get_area(b, b->set_faces[aux + j]);
            total += b->face_area[j];
        }
        for (int j = 0; j < b->set_size[s]; ++j) {
            const double w = b->face_area[j] / (3 * total);
            double tr[3];
            for (int c = 0; c < 3; ++c) tr[c] = w * b->set_f[3 * s + c]; /* resize2 */
            double *ff = b->face_f + 9 * (size_t)b->set_faces[aux + j];
            for (int k = 0; k < 3; ++k) /* Face::add_force_to_node(0..2, traction) */
                for (int c = 0; c < 3; ++c) ff[3 * k + c] += tr[c];
        }
        aux += b->set_size[s];
    }
}

int orc_blob_update_internal_forces(orc_blob *b) {
    int num_inversions = 0;
    apply_ctforces(b);
    const int nomass = b->solver == ORC_NOMASS_CG;
#pragma omp parallel num_threads(b->nthreads) reduction(+ : num_inversions)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
#pragma omp for schedule(guided)
        for (int e = 0; e < b->T; ++e) {
            double J[3][3], S[3][3] = {{0}}, du[12];
            elem_jacobian(b, e, J);
            if (elem_dpsi_vol(b, e, J)) num_inversions++;
            elem_viscosity(b, e);
            elem_shear_stress(b, e, J, S);
            elem_bulk_stress(b, e, S);
            if (b->calc_noise == 1) elem_fluct_stress(b, e, S, &b->rng[tid]);
            /* mat3_double_contraction_symmetric, src/mat_vec_fns.cpp:108-111 */
            b->stress_mag[e] = sqrt(S[0][0] * S[0][0] + S[1][1] * S[1][1] + S[2][2] * S[2][2] +
                                    2 * (S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][2] * S[1][2]));
            const int *t = b->tet + 10 * (size_t)e;
            if (!nomass) {
                /* get_element_velocity_vector :448-463 + mat12_apply (src/mat_vec_fns.cpp:28-36) */
                double v[12], tmp[12];
                for (int a = 0; a < 4; ++a)
                    for (int i = 0; i < 3; ++i) v[4 * i + a] = b->vel[3 * (size_t)t[a] + i];
                const double *V = b->visc + 144 * (size_t)e;
                for (int i = 0; i < 12; ++i) {
                    tmp[i] = 0;
                    for (int j = 0; j < 12; ++j) tmp[i] += V[12 * i + j] * v[j];
                }
                for (int i = 0; i < 12; ++i) du[i] = tmp[i];
            } else {
                for (int i = 0; i < 12; ++i) du[i] = 0;
            }
            /* apply_stress_tensor :436-443 */
            const double *dpsi = b->dpsi + 12 * (size_t)e;
            const double vol = b->vol[e];
            for (int i = 0; i < 3; ++i) {
                du[4 * i] += vol * (dpsi[0] * S[i][0] + dpsi[4] * S[i][1] + dpsi[8] * S[i][2]);
                du[4 * i + 1] += vol * (dpsi[1] * S[i][0] + dpsi[5] * S[i][1] + dpsi[9] * S[i][2]);
                du[4 * i + 2] += vol * (dpsi[2] * S[i][0] + dpsi[6] * S[i][1] + dpsi[10] * S[i][2]);
                du[4 * i + 3] += vol * (dpsi[3] * S[i][0] + dpsi[7] * S[i][1] + dpsi[11] * S[i][2]);
            }
            /* add_element_force_vector :468-483 */
            double *nf = b->node_force + 30 * (size_t)e;
            for (int a = 0; a < 4; ++a)
                for (int i = 0; i < 3; ++i) nf[3 * a + i] -= du[4 * i + a];
        }
    }
    return num_inversions ? ORC_EINVERTED : ORC_OK;
}

/* ---------------------------------------------------------------------------
 * solvers
 * ------------------------------------------------------------------------- */

/* SparseMatrixFixedPattern::build (src/SparseMatrixFixedPattern.cpp:86-94) with
 * sparse_entry_sources::sum_all_sources (src/SparseMatrixTypes.cpp:40-46) */
static void nomass_build(orc_blob *b) {
#pragma omp parallel for num_threads(b->nthreads)
    for (int k = 0; k < b->nnz; ++k) {
        double sum = 0.0;
        for (int s = b->sptr[k]; s < b->sptr[k + 1]; ++s) sum += *(b->src[s]);
        b->entry[k].val = sum;
    }
}

/* SparseMatrixFixedPattern::apply(vector<arr3>) :148-187 */
static void nomass_apply(orc_blob *b, const double *in, double *out) {
    const int rows = b->rows;
#pragma omp parallel num_threads(b->nthreads)
    {
#pragma omp for
        for (int i = 0; i < rows; ++i) b->work_in[i] = in[i];
#pragma omp for
        for (int i = 0; i < rows; ++i) {
            b->work_out[i] = 0.0;
            for (int j = b->key[i]; j < b->key[i + 1]; ++j) b->work_out[i] += b->entry[j].val * b->work_in[b->entry[j].col];
        }
#pragma omp for
        for (int i = 0; i < rows; ++i) out[i] = b->work_out[i];
    }
}

/* NoMassCGSolver::solve and helpers, src/NoMassCGSolver.cpp:156-281 */
static int nomass_solve(orc_blob *b, double *x) {
    const int n = b->n;
    double *r = b->r, *p = b->p, *z = b->z, *q = b->q, *f = b->f, *M = b->precond;
    nomass_build(b);
    for (int i = 0; i < b->rows; ++i) M[i] = 1.0 / *(b->diag[i]); /* calc_inverse_diagonal :305-312 */
    double delta_new = 0;
#pragma omp parallel for num_threads(b->nthreads) reduction(+ : delta_new)
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            r[3 * i + c] = x[3 * i + c];
            f[3 * i + c] = x[3 * i + c];
            x[3 * i + c] = 0;
            z[3 * i + c] = M[3 * i + c] * r[3 * i + c];
            p[3 * i + c] = z[3 * i + c];
        }
        delta_new += r[3 * i] * z[3 * i] + r[3 * i + 1] * z[3 * i + 1] + r[3 * i + 2] * z[3 * i + 2];
    }
    for (int it = 0; it < b->imax; ++it) {
        nomass_apply(b, p, q);
        double pTq = 0;
#pragma omp parallel for num_threads(b->nthreads) reduction(+ : pTq)
        for (int i = 0; i < n; ++i) pTq += p[3 * i] * q[3 * i] + p[3 * i + 1] * q[3 * i + 1] + p[3 * i + 2] * q[3 * i + 2];
        const double alpha = delta_new / pTq;
        /* vec3_add_to_scaled, src/mat_vec_fns.cpp:187-197 */
#pragma omp parallel for num_threads(b->nthreads)
        for (int i = 0; i < 3 * n; ++i) x[i] += alpha * p[i];
        const double malpha = -alpha;
#pragma omp parallel for num_threads(b->nthreads)
        for (int i = 0; i < 3 * n; ++i) r[i] += malpha * q[i];
        double r2 = 0, f2 = 0;
#pragma omp parallel for num_threads(b->nthreads) reduction(+ : r2, f2)
        for (int i = 0; i < n; ++i) {
            r2 += r[3 * i] * r[3 * i] + r[3 * i + 1] * r[3 * i + 1] + r[3 * i + 2] * r[3 * i + 2];
            f2 += f[3 * i] * f[3 * i] + f[3 * i + 1] * f[3 * i + 1] + f[3 * i + 2] * f[3 * i + 2];
        }
        const double res2 = (f2 == 0.0) ? 0.0 : r2 / f2;
        if (res2 < b->eps2) {
            b->last_iters = it + 1;
            b->total_iters += it + 1;
            return ORC_OK;
        }
        const double delta_old = delta_new;
        delta_new = 0;
#pragma omp parallel for num_threads(b->nthreads) reduction(+ : delta_new)
        for (int i = 0; i < n; ++i) {
            z[3 * i] = M[3 * i] * r[3 * i];
            z[3 * i + 1] = M[3 * i + 1] * r[3 * i + 1];
            z[3 * i + 2] = M[3 * i + 2] * r[3 * i + 2];
            delta_new += r[3 * i] * z[3 * i] + r[3 * i + 1] * z[3 * i + 1] + r[3 * i + 2] * z[3 * i + 2];
        }
        const double beta = delta_new / delta_old;
        /* vec3_scale_and_add :202-212 */
#pragma omp parallel for num_threads(b->nthreads)
        for (int i = 0; i < 3 * n; ++i) p[i] = beta * p[i] + z[i];
    }
    b->last_iters = b->imax;
    b->total_iters += b->imax;
    return ORC_ECGMAXIT;
}

/* ConjugateGradientSolver::solve and helpers, src/ConjugateGradientSolver.cpp:193-334 */
static int cg_solve(orc_blob *b, double *x) {
    const int n = b->n;
    double *r = b->r, *d = b->d, *q = b->q, *s = b->s, *f = b->f, *M = b->precond;
    double delta_new = 0;
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            r[3 * i + c] = x[3 * i + c];
            f[3 * i + c] = x[3 * i + c];
            x[3 * i + c] = 0;
            d[3 * i + c] = M[i] * r[3 * i + c];
        }
        delta_new += r[3 * i] * d[3 * i] + r[3 * i + 1] * d[3 * i + 1] + r[3 * i + 2] * d[3 * i + 2];
    }
    for (int it = 0; it < b->imax; ++it) {
        double r2 = 0, f2 = 0;
        for (int i = 0; i < n; ++i) {
            r2 += r[3 * i] * r[3 * i] + r[3 * i + 1] * r[3 * i + 1] + r[3 * i + 2] * r[3 * i + 2];
            f2 += f[3 * i] * f[3 * i] + f[3 * i + 1] * f[3 * i + 1] + f[3 * i + 2] * f[3 * i + 2];
        }
        const double res2 = (f2 == 0.0) ? 0.0 : r2 / f2;
        if (res2 < b->eps2) {
            b->last_iters = it;
            b->total_iters += it;
            return ORC_OK;
        }
        double dTq = 0;
        for (int i = 0; i < n; ++i) {
            q[3 * i] = 0; q[3 * i + 1] = 0; q[3 * i + 2] = 0;
            for (int j = b->mkey[i]; j < b->mkey[i + 1]; ++j) {
                const int c = b->mentry[j].col;
                q[3 * i] += b->mentry[j].val * d[3 * c];
                q[3 * i + 1] += b->mentry[j].val * d[3 * c + 1];
                q[3 * i + 2] += b->mentry[j].val * d[3 * c + 2];
            }
            dTq += d[3 * i] * q[3 * i] + d[3 * i + 1] * q[3 * i + 1] + d[3 * i + 2] * q[3 * i + 2];
        }
        const double alpha = delta_new / dTq;
        for (int i = 0; i < 3 * n; ++i) x[i] += alpha * d[i];
        const double malpha = -alpha;
        for (int i = 0; i < 3 * n; ++i) r[i] += malpha * q[i];
        const double delta_old = delta_new;
        delta_new = 0;
        for (int i = 0; i < n; ++i) {
            s[3 * i] = M[i] * r[3 * i];
            s[3 * i + 1] = M[i] * r[3 * i + 1];
            s[3 * i + 2] = M[i] * r[3 * i + 2];
            delta_new += r[3 * i] * s[3 * i] + r[3 * i + 1] * s[3 * i + 1] + r[3 * i + 2] * s[3 * i + 2];
        }
        const double beta = delta_new / delta_old;
        for (int i = 0; i < 3 * n; ++i) d[i] = s[i] + beta * d[i];
    }
    b->last_iters = b->imax;
    b->total_iters += b->imax;
    return ORC_ECGMAXIT;
}

/* MassLumpedSolver::solve, src/MassLumpedSolver.cpp:65-72 */
static void lumped_solve(orc_blob *b, double *x) {
    for (int i = 0; i < b->n; ++i) {
        x[3 * i] = x[3 * i] * b->inv_m[i];
        x[3 * i + 1] = x[3 * i + 1] * b->inv_m[i];
        x[3 * i + 2] = x[3 * i + 2] * b->inv_m[i];
    }
}

/* ---------------------------------------------------------------------------
 * Blob step
 * ------------------------------------------------------------------------- */

/* Blob::zero_force + Blob::set_forces_to_zero, src/Blob.cpp:1745-1760 */
void orc_blob_zero_forces(orc_blob *b) {
    memset(b->node_force, 0, sizeof(double) * 30 * (size_t)b->T);
    memset(b->force, 0, sizeof(double) * 3 * (size_t)b->n);
    if (b->face_f) memset(b->face_f, 0, sizeof(double) * 9 * (size_t)b->n_faces);
}

/* tetra_element_linear::linearise_element, src/tetra_element_linear.cpp:553-577 */
static void linearise_elements(orc_blob *b) {
    static const int mid[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    for (int e = 0; e < b->T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int m = 0; m < 6; ++m) {
            double *pm = b->pos + 3 * (size_t)t[4 + m];
            const double *pa = b->pos + 3 * (size_t)t[mid[m][0]], *pb = b->pos + 3 * (size_t)t[mid[m][1]];
            for (int c = 0; c < 3; ++c) pm[c] = .5 * (pa[c] + pb[c]);
        }
    }
}

/* Blob::aggregate_forces_and_solve, src/Blob.cpp:3147-3244 */
static int aggregate_forces_and_solve(orc_blob *b) {
    const int n = b->n;
#pragma omp parallel for num_threads(b->nthreads) schedule(guided)
    for (int i = 0; i < n; ++i) {
        for (int m = b->cptr[i]; m < b->cptr[i + 1]; ++m) {
            b->force[3 * i] += b->contrib[m][0];
            b->force[3 * i + 1] += b->contrib[m][1];
            b->force[3 * i + 2] += b->contrib[m][2];
        }
    }
    /* surface forces onto nodes, face order (a face's fourth, opposite node always receives zero here) */
    for (int f = 0; f < b->n_faces; ++f)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) b->force[3 * (size_t)b->face_nodes[3 * f + k] + c] += b->face_f[9 * f + 3 * k + c];
    if (b->calc_stokes == 1) {
        const int nomass = b->solver == ORC_NOMASS_CG;
        if (!nomass || b->calc_noise == 1) {
#pragma omp parallel num_threads(b->nthreads)
            {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
#pragma omp for schedule(guided)
                for (int i = 0; i < n; ++i) {
                    double *fi = b->force + 3 * (size_t)i;
                    if (!nomass) {
                        fi[0] -= b->vel[3 * i] * b->stokes_drag[i];
                        fi[1] -= b->vel[3 * i + 1] * b->stokes_drag[i];
                        fi[2] -= b->vel[3 * i + 2] * b->stokes_drag[i];
                    }
                    if (b->calc_noise == 1) {
                        fi[0] -= rand_half(&b->rng[tid]) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                        fi[1] -= rand_half(&b->rng[tid]) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                        fi[2] -= rand_half(&b->rng[tid]) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                    }
                }
            }
        }
    }
    /* Blob::linearise_force, src/Blob.cpp:781-799 */
    for (int e = 0; e < b->T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        double *F = b->force;
        for (int j = 0; j < 3; ++j) {
            F[3 * t[0] + j] += 0.5 * (F[3 * t[4] + j] + F[3 * t[5] + j] + F[3 * t[6] + j]);
            F[3 * t[1] + j] += 0.5 * (F[3 * t[4] + j] + F[3 * t[7] + j] + F[3 * t[8] + j]);
            F[3 * t[2] + j] += 0.5 * (F[3 * t[5] + j] + F[3 * t[7] + j] + F[3 * t[9] + j]);
            F[3 * t[3] + j] += 0.5 * (F[3 * t[6] + j] + F[3 * t[8] + j] + F[3 * t[9] + j]);
        }
        for (int j = 4; j < 10; ++j) F[3 * t[j]] = F[3 * t[j] + 1] = F[3 * t[j] + 2] = 0.;
    }
    for (int k = 0; k < b->npinned; ++k) {
        const int pn = b->pinned[k];
        b->force[3 * pn] = b->force[3 * pn + 1] = b->force[3 * pn + 2] = 0;
    }
    memcpy(b->rhs, b->force, sizeof(double) * 3 * (size_t)n);
    if (b->solver == ORC_NOMASS_CG) return nomass_solve(b, b->force);
    if (b->solver == ORC_CG) return cg_solve(b, b->force);
    lumped_solve(b, b->force);
    return ORC_OK;
}

/* Blob::euler_integrate, src/Blob.cpp:3249-3279 */
static void euler_integrate(orc_blob *b) {
    const int n = b->n;
    const double dt = b->dt;
    if (b->solver == ORC_NOMASS_CG) {
#pragma omp parallel for num_threads(b->nthreads) schedule(static)
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) {
                b->vel[3 * i + c] = b->force[3 * i + c];
                b->pos[3 * i + c] += b->force[3 * i + c] * dt;
            }
    } else {
#pragma omp parallel for num_threads(b->nthreads) schedule(static)
        for (int i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) b->vel[3 * i + c] += b->force[3 * i + c] * dt;
            for (int c = 0; c < 3; ++c) b->pos[3 * i + c] += b->vel[3 * i + c] * dt;
        }
    }
}

/* Blob::update_positions, src/Blob.cpp:493-508 */
int orc_blob_update_positions(orc_blob *b) {
    int st = aggregate_forces_and_solve(b);
    if (st != ORC_OK) return st;
    euler_integrate(b);
    linearise_elements(b);
    return ORC_OK;
}

/* the per-blob slice of World::run, src/World.cpp:1788,1862,2037,2058 */
int orc_blob_step(orc_blob *b, int nsteps) {
    for (int s = 0; s < nsteps; ++s) {
        orc_blob_zero_forces(b);
        int st = orc_blob_update_internal_forces(b);
        if (st != ORC_OK) return st;
        st = orc_blob_update_positions(b);
        if (st != ORC_OK) return st;
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------------------
 * initialisation -- Blob::init (src/Blob.cpp:161-365)
 * ------------------------------------------------------------------------- */

/* mat3_invert, src/mat_vec_fns.cpp:125-154 */
static void mat3_invert(double m[3][3], double *inv) {
    inv[0] = m[2][2] * m[1][1] - m[2][1] * m[1][2];
    inv[1] = m[2][1] * m[0][2] - m[2][2] * m[0][1];
    inv[2] = m[1][2] * m[0][1] - m[1][1] * m[0][2];
    inv[3] = m[2][0] * m[1][2] - m[2][2] * m[1][0];
    inv[4] = m[2][2] * m[0][0] - m[2][0] * m[0][2];
    inv[5] = m[1][0] * m[0][2] - m[1][2] * m[0][0];
    inv[6] = m[2][1] * m[1][0] - m[2][0] * m[1][1];
    inv[7] = m[2][0] * m[0][1] - m[2][1] * m[0][0];
    inv[8] = m[1][1] * m[0][0] - m[1][0] * m[0][1];
    double det = m[0][0] * inv[0] + m[1][0] * inv[1] + m[2][0] * inv[2];
    det = 1.0 / det;
    for (int i = 0; i < 9; ++i) inv[i] *= det;
}

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/*
 * NoMassCGSolver::init pattern (src/NoMassCGSolver.cpp:56-153) built through
 * SparsityPattern (src/SparsityPattern.cpp:35-110). The reference inserts
 * each source into a column-sorted list per row; the resulting matrix is:
 * per row, columns ascending; per entry, sources in registration order. For
 * a conforming mesh the registration order of one entry is: the identity
 * source `one` (only for pinned or midpoint nodes, and only if no element
 * source reached that diagonal first), then one source per element that
 * holds both nodes at vertex slots, in element order, then the node's Stokes
 * drag. This builds that structure directly instead of by list insertion.
 */
static int nomass_init(orc_blob *b) {
    const int n = b->n, T = b->T;
    b->rows = 3 * n;
    b->one = 1;
    /* first element where each node gets an element source / an identity candidate */
    int *e0 = malloc(sizeof(int) * n), *e1 = malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) e0[i] = e1[i] = T;
    for (int e = T - 1; e >= 0; --e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int s = 0; s < 10; ++s) {
            const int X = t[s];
            if (s < 4 && !b->is_pinned[X]) e0[X] = e;
            if (s >= 4 || b->is_pinned[X]) e1[X] = e;
        }
    }
    /* block neighbours per node (unpinned vertex pairs sharing an element) */
    int *ncnt = xcalloc(n + 1, sizeof(int));
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 4; ++a)
            if (!b->is_pinned[t[a]])
                for (int c = 0; c < 4; ++c)
                    if (!b->is_pinned[t[c]]) ncnt[t[a]]++;
    }
    int *nptr = malloc(sizeof(int) * (n + 1));
    nptr[0] = 0;
    for (int i = 0; i < n; ++i) nptr[i + 1] = nptr[i] + ncnt[i];
    int *nb = malloc(sizeof(int) * (size_t)(nptr[n] ? nptr[n] : 1));
    for (int i = 0; i < n; ++i) ncnt[i] = 0;
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 4; ++a)
            if (!b->is_pinned[t[a]])
                for (int c = 0; c < 4; ++c)
                    if (!b->is_pinned[t[c]]) nb[nptr[t[a]] + ncnt[t[a]]++] = t[c];
    }
    int *uptr = malloc(sizeof(int) * (n + 1)); /* unique neighbours, sorted */
    uptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        int *L = nb + nptr[i];
        int m = nptr[i + 1] - nptr[i];
        qsort(L, m, sizeof(int), cmp_int);
        int u = 0;
        for (int k = 0; k < m; ++k)
            if (u == 0 || L[u - 1] != L[k]) L[u++] = L[k];
        ncnt[i] = u;
    }
    for (int i = 0; i < n; ++i) uptr[i + 1] = uptr[i] + ncnt[i];
    int *un = malloc(sizeof(int) * (size_t)(uptr[n] ? uptr[n] : 1));
    for (int i = 0; i < n; ++i) memcpy(un + uptr[i], nb + nptr[i], sizeof(int) * ncnt[i]);
    free(nb);
    free(nptr);
    /* rows: node X row i has 3 entries per block neighbour, or one identity entry */
    b->key = malloc(sizeof(int) * (b->rows + 1));
    int nnz = 0;
    for (int X = 0; X < n; ++X) {
        int nblk = uptr[X + 1] - uptr[X];
        int has_one = e1[X] < e0[X];
        if (nblk == 0 && !has_one) { /* node in no element: reference diagonal pointer undefined */
            free(e0); free(e1); free(ncnt); free(uptr); free(un);
            return ORC_EINPUT;
        }
        for (int i = 0; i < 3; ++i) {
            b->key[3 * X + i] = nnz;
            nnz += nblk ? 3 * nblk : 1;
        }
    }
    b->key[b->rows] = nnz;
    b->nnz = nnz;
    b->entry = malloc(sizeof(orc_entry) * (size_t)nnz);
    b->sptr = xcalloc((size_t)nnz + 1, sizeof(int));
    b->diag = malloc(sizeof(double *) * b->rows);
    for (int X = 0; X < n; ++X) {
        int nblk = uptr[X + 1] - uptr[X];
        for (int i = 0; i < 3; ++i) {
            int k = b->key[3 * X + i];
            if (nblk == 0) {
                b->entry[k].col = 3 * X + i;
                b->entry[k].val = 0;
            } else {
                for (int m = 0; m < nblk; ++m)
                    for (int j = 0; j < 3; ++j) {
                        b->entry[k + 3 * m + j].col = 3 * un[uptr[X] + m] + j;
                        b->entry[k + 3 * m + j].val = 0;
                    }
            }
        }
    }
    /* source counts per entry */
    int *cnt = xcalloc((size_t)nnz + 1, sizeof(int));
#define ENTRY_OF(Xn, i, Yn, j, out)                                                   \
    do {                                                                              \
        const int *L_ = un + uptr[Xn];                                                \
        int lo_ = 0, hi_ = uptr[(Xn) + 1] - uptr[Xn] - 1;                             \
        while (lo_ < hi_) {                                                           \
            int mid_ = (lo_ + hi_) >> 1;                                              \
            if (L_[mid_] < (Yn)) lo_ = mid_ + 1; else hi_ = mid_;                     \
        }                                                                             \
        out = b->key[3 * (Xn) + (i)] + 3 * lo_ + (j);                                 \
    } while (0)
    for (int X = 0; X < n; ++X) {
        if (e1[X] < e0[X])
            for (int i = 0; i < 3; ++i) {
                int k;
                if (uptr[X + 1] > uptr[X]) ENTRY_OF(X, i, X, i, k); else k = b->key[3 * X + i];
                cnt[k]++;
            }
        if (b->calc_stokes == 1 && !b->is_pinned[X])
            for (int i = 0; i < 3; ++i) {
                int k;
                if (uptr[X + 1] > uptr[X]) ENTRY_OF(X, i, X, i, k); else k = b->key[3 * X + i];
                cnt[k]++;
            }
    }
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 4; ++a) {
            if (b->is_pinned[t[a]]) continue;
            for (int c = 0; c < 4; ++c) {
                if (b->is_pinned[t[c]]) continue;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        int k;
                        ENTRY_OF(t[a], i, t[c], j, k);
                        cnt[k]++;
                    }
            }
        }
    }
    for (int k = 0; k < nnz; ++k) b->sptr[k + 1] = b->sptr[k] + cnt[k];
    b->src = malloc(sizeof(double *) * (size_t)(b->sptr[nnz] ? b->sptr[nnz] : 1));
    for (int k = 0; k < nnz; ++k) cnt[k] = 0;
    /* fill: identity first, then elements in order, then Stokes */
    for (int X = 0; X < n; ++X)
        if (e1[X] < e0[X])
            for (int i = 0; i < 3; ++i) {
                int k;
                if (uptr[X + 1] > uptr[X]) ENTRY_OF(X, i, X, i, k); else k = b->key[3 * X + i];
                b->src[b->sptr[k] + cnt[k]++] = &b->one;
            }
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 4; ++a) {
            if (b->is_pinned[t[a]]) continue;
            for (int c = 0; c < 4; ++c) {
                if (b->is_pinned[t[c]]) continue;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        int k;
                        ENTRY_OF(t[a], i, t[c], j, k);
                        b->src[b->sptr[k] + cnt[k]++] = &b->visc[144 * (size_t)e + 12 * (a + 4 * i) + (c + 4 * j)];
                    }
            }
        }
    }
    if (b->calc_stokes == 1)
        for (int X = 0; X < n; ++X)
            if (!b->is_pinned[X])
                for (int i = 0; i < 3; ++i) {
                    int k;
                    if (uptr[X + 1] > uptr[X]) ENTRY_OF(X, i, X, i, k); else k = b->key[3 * X + i];
                    b->src[b->sptr[k] + cnt[k]++] = &b->stokes_drag[X];
                }
#undef ENTRY_OF
    /* SparseMatrixFixedPattern::init diagonal pointers, src/SparseMatrixFixedPattern.cpp:56-62 */
    for (int r = 0; r < b->rows; ++r)
        for (int k = b->key[r]; k < b->key[r + 1]; ++k)
            if (b->entry[k].col == r) b->diag[r] = &b->entry[k].val;
    free(cnt);
    free(e0);
    free(e1);
    free(ncnt);
    free(uptr);
    free(un);
    b->precond = xcalloc(b->rows, sizeof(double));
    return ORC_OK;
}

/*
 * ConjugateGradientSolver::init (src/ConjugateGradientSolver.cpp:51-191). The
 * reference accumulates a dense n x n matrix, then keeps its non-zero entries
 * row by row in column order. Here the same sums are accumulated per row in
 * element order into a sorted neighbour list.
 */
static int cg_init(orc_blob *b) {
    const int n = b->n, T = b->T;
    /* neighbour lists of all nodes with element (vertex) pairs and diagonals */
    int *cnt = xcalloc(n + 1, sizeof(int));
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 10; ++a)
            for (int c = 0; c < 10; ++c)
                if ((a < 4 && c < 4) || a == c) cnt[t[a]]++;
    }
    int *ptr = malloc(sizeof(int) * (n + 1));
    ptr[0] = 0;
    for (int i = 0; i < n; ++i) ptr[i + 1] = ptr[i] + cnt[i];
    int *nb = malloc(sizeof(int) * (size_t)(ptr[n] ? ptr[n] : 1));
    for (int i = 0; i < n; ++i) cnt[i] = 0;
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 10; ++a)
            for (int c = 0; c < 10; ++c)
                if ((a < 4 && c < 4) || a == c) nb[ptr[t[a]] + cnt[t[a]]++] = t[c];
    }
    int *uptr = malloc(sizeof(int) * (n + 1));
    uptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        int *L = nb + ptr[i];
        int m = ptr[i + 1] - ptr[i], u = 0;
        qsort(L, m, sizeof(int), cmp_int);
        for (int k = 0; k < m; ++k)
            if (u == 0 || L[u - 1] != L[k]) L[u++] = L[k];
        cnt[i] = u;
        uptr[i + 1] = uptr[i] + u;
    }
    int *cols = malloc(sizeof(int) * (size_t)(uptr[n] ? uptr[n] : 1));
    double *vals = xcalloc((size_t)uptr[n] + 1, sizeof(double));
    for (int i = 0; i < n; ++i) memcpy(cols + uptr[i], nb + ptr[i], sizeof(int) * cnt[i]);
    free(nb);
    free(ptr);
    for (int e = 0; e < T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int a = 0; a < 10; ++a)
            for (int c = 0; c < 10; ++c) {
                const int ni = t[a], nj = t[c];
                if (!((a < 4 && c < 4) || a == c)) continue;
                int lo = uptr[ni], hi = uptr[ni + 1] - 1;
                while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (cols[mid] < nj) lo = mid + 1; else hi = mid;
                }
                double *v = &vals[lo];
                if (a < 4 && c < 4) {
                    if (!b->is_pinned[ni] && !b->is_pinned[nj]) {
                        if (a == c) *v += .1 * b->rho[e] * b->vol0[e];
                        else *v += .05 * b->rho[e] * b->vol0[e];
                    } else if (a == c) {
                        *v = 1;
                    }
                } else if (a == c) {
                    *v = 1;
                }
            }
    }
    b->mkey = malloc(sizeof(int) * (n + 1));
    int nz = 0;
    for (int i = 0; i < n; ++i) {
        b->mkey[i] = nz;
        for (int k = uptr[i]; k < uptr[i + 1]; ++k)
            if (vals[k] != 0) nz++;
    }
    b->mkey[n] = nz;
    b->mnnz = nz;
    b->mentry = malloc(sizeof(orc_entry) * (size_t)(nz ? nz : 1));
    b->precond = xcalloc(n, sizeof(double));
    nz = 0;
    for (int i = 0; i < n; ++i) {
        double dg = 0;
        for (int k = uptr[i]; k < uptr[i + 1]; ++k) {
            if (cols[k] == i) dg = vals[k];
            if (vals[k] != 0) { b->mentry[nz].col = cols[k]; b->mentry[nz].val = vals[k]; nz++; }
        }
        b->precond[i] = 1.0 / dg;
    }
    free(cnt);
    free(uptr);
    free(cols);
    free(vals);
    b->d = xcalloc(3 * (size_t)n, sizeof(double));
    b->s = xcalloc(3 * (size_t)n, sizeof(double));
    return ORC_OK;
}

/* MassLumpedSolver::init, src/MassLumpedSolver.cpp:27-62 */
static int lumped_init(orc_blob *b) {
    b->inv_m = xcalloc(b->n, sizeof(double));
    for (int e = 0; e < b->T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        for (int i = 0; i < 10; ++i) {
            if (i < 4) b->inv_m[t[i]] += .25 * b->rho[e] * b->vol0[e];
            else b->inv_m[t[i]] = 1;
        }
    }
    for (int k = 0; k < b->npinned; ++k) b->inv_m[b->pinned[k]] = 1.0;
    for (int i = 0; i < b->n; ++i) b->inv_m[i] = 1.0 / b->inv_m[i];
    return ORC_OK;
}

orc_blob *orc_blob_create(int n_nodes, const double *pos, double scale_m, int n_elem, const int *tets,
                          const double *mat6, const double *stokes_radius, int n_pinned, const int *pinned,
                          const orc_params *p, int solver, int n_threads, int *status) {
    *status = ORC_EINPUT;
    if (n_nodes <= 0 || n_elem <= 0 || n_threads <= 0 || solver < 0 || solver > 2) return NULL;
    for (size_t i = 0; i < 10 * (size_t)n_elem; ++i)
        if (tets[i] < 0 || tets[i] >= n_nodes) return NULL;
    for (int i = 0; i < n_pinned; ++i)
        if (pinned[i] < 0 || pinned[i] >= n_nodes) return NULL;
    orc_blob *b = xcalloc(1, sizeof(orc_blob));
    const int n = n_nodes, T = n_elem;
    b->n = n;
    b->T = T;
    b->solver = solver;
    b->nthreads = n_threads;
    /* SimulationParams::assign, src/SimulationParams.cpp:252-265,415-421,531-537 */
    b->dt = p->dt / MESO_TIME;
    b->kT = p->kT / MESO_ENERGY;
    b->eps2 = p->epsilon;
    b->eps2 *= b->eps2;
    b->stokes_visc = p->stokes_visc / (MESO_PRESSURE * MESO_TIME);
    b->imax = p->max_iterations_cg;
    b->calc_noise = p->calc_noise;
    b->calc_stokes = p->calc_stokes;
    /* World: scale /= mesoDimensions::length (src/World.cpp:2632); Blob::load_nodes :1978-1980 */
    const double scale = scale_m / MESO_LENGTH;
    b->pos = malloc(sizeof(double) * 3 * (size_t)n);
    b->vel = xcalloc(3 * (size_t)n, sizeof(double));
    b->force = xcalloc(3 * (size_t)n, sizeof(double));
    b->rhs = xcalloc(3 * (size_t)n, sizeof(double));
    b->stokes_radius = malloc(sizeof(double) * n);
    b->stokes_drag = xcalloc(n, sizeof(double));
    for (size_t i = 0; i < 3 * (size_t)n; ++i) b->pos[i] = scale * pos[i];
    for (int i = 0; i < n; ++i) b->stokes_radius[i] = stokes_radius[i] * scale; /* load_stokes_params :2335 */
    b->tet = malloc(sizeof(int) * 10 * (size_t)T);
    memcpy(b->tet, tets, sizeof(int) * 10 * (size_t)T);
    b->rho = malloc(sizeof(double) * T); b->A = malloc(sizeof(double) * T); b->B = malloc(sizeof(double) * T);
    b->G = malloc(sizeof(double) * T); b->E = malloc(sizeof(double) * T);
    /* Blob::load_material_params :2275-2283, including the second-viscosity unit mix of :2281 */
    for (int e = 0; e < T; ++e) {
        const double *m = mat6 + 6 * (size_t)e;
        b->rho[e] = m[0] * MESO_VOLUME / MESO_MASS;
        b->A[e] = m[1] / (MESO_PRESSURE * MESO_TIME);
        b->B[e] = m[2] / (MESO_PRESSURE * MESO_TIME) - (2.0 / 3.0) * m[1];
        b->G[e] = m[3] / MESO_PRESSURE;
        b->E[e] = m[4] / MESO_PRESSURE;
    }
    b->vol0 = xcalloc(T, sizeof(double)); b->vol = xcalloc(T, sizeof(double));
    b->last_det = xcalloc(T, sizeof(double));
    b->jinv0 = xcalloc(9 * (size_t)T, sizeof(double));
    b->dpsi = xcalloc(12 * (size_t)T, sizeof(double));
    b->visc = xcalloc(144 * (size_t)T, sizeof(double));
    b->node_force = xcalloc(30 * (size_t)T, sizeof(double));
    b->F = xcalloc(9 * (size_t)T, sizeof(double));
    b->stress_mag = xcalloc(T, sizeof(double));
    b->is_pinned = xcalloc(n, sizeof(int));
    b->npinned = n_pinned;
    b->pinned = malloc(sizeof(int) * (n_pinned ? n_pinned : 1));
    for (int i = 0; i < n_pinned; ++i) { b->pinned[i] = pinned[i]; b->is_pinned[pinned[i]] = 1; }
    /* Blob::init: linearise, rest state, connectivity, solver (src/Blob.cpp:202-247) */
    linearise_elements(b);
    for (int e = 0; e < T; ++e) { /* calc_rest_state_info :3080-3143 */
        double J[3][3];
        elem_jacobian(b, e, J);
        mat3_invert(J, b->jinv0 + 9 * (size_t)e);
        elem_dpsi_vol(b, e, J);
        b->vol0[e] = b->vol[e];
    }
    /* calculate_node_element_connectivity :3284-3314 */
    b->cptr = xcalloc((size_t)n + 1, sizeof(int));
    for (size_t i = 0; i < 10 * (size_t)T; ++i) b->cptr[tets[i] + 1]++;
    for (int i = 0; i < n; ++i) b->cptr[i + 1] += b->cptr[i];
    b->contrib = malloc(sizeof(double *) * 10 * (size_t)T);
    b->contrib_es = malloc(sizeof(int) * 10 * (size_t)T);
    int *fill = xcalloc(n, sizeof(int));
    for (int e = 0; e < T; ++e)
        for (int j = 0; j < 10; ++j) {
            const int X = tets[10 * (size_t)e + j];
            const int k = b->cptr[X] + fill[X]++;
            b->contrib[k] = b->node_force + 30 * (size_t)e + 3 * j;
            b->contrib_es[k] = 10 * e + j;
        }
    free(fill);
    b->r = xcalloc(3 * (size_t)n, sizeof(double)); b->p = xcalloc(3 * (size_t)n, sizeof(double));
    b->z = xcalloc(3 * (size_t)n, sizeof(double)); b->q = xcalloc(3 * (size_t)n, sizeof(double));
    b->f = xcalloc(3 * (size_t)n, sizeof(double));
    b->work_in = xcalloc(3 * (size_t)n, sizeof(double));
    b->work_out = xcalloc(3 * (size_t)n, sizeof(double));
    int st = ORC_OK;
    if (solver == ORC_NOMASS_CG) {
        /* NoMassCGSolver::init recomputes J, dpsi, vol and the viscosity matrix (:78-81) */
        for (int e = 0; e < T; ++e) {
            double J[3][3];
            elem_jacobian(b, e, J);
            elem_dpsi_vol(b, e, J);
            elem_viscosity(b, e);
        }
        st = nomass_init(b);
    } else if (solver == ORC_CG) {
        st = cg_init(b);
    } else {
        st = lumped_init(b);
    }
    if (st != ORC_OK) { orc_blob_destroy(b); *status = st; return NULL; }
    /* Stokes drag, Blob::init :262-268 */
    if (b->calc_stokes == 1)
        for (int i = 0; i < n; ++i) b->stokes_drag[i] = 6.0 * FFEA_PI * b->stokes_visc * b->stokes_radius[i];
    /* one RngStream per thread, created from the package seed */
    b->rng = malloc(sizeof(orc_rng) * n_threads);
    for (int t = 0; t < n_threads; ++t) orc_rng_create(&b->rng[t]);
    *status = ORC_OK;
    return b;
}

void orc_blob_destroy(orc_blob *b) {
    if (!b) return;
    void *ptrs[] = {b->pos, b->vel, b->force, b->rhs, b->stokes_radius, b->stokes_drag, b->is_pinned, b->pinned,
                    b->tet, b->rho, b->A, b->B, b->G, b->E, b->vol0, b->vol, b->last_det, b->jinv0, b->dpsi,
                    b->visc, b->node_force, b->F, b->stress_mag, b->cptr, b->contrib, b->contrib_es, b->key,
                    b->entry, b->sptr, b->src, b->diag, b->precond, b->r, b->p, b->z, b->q, b->f, b->work_in,
                    b->work_out, b->mkey, b->mentry, b->d, b->s, b->inv_m, b->rng, b->lctf_node, b->set_size,
                    b->set_faces, b->face_nodes, b->lctf_f, b->set_f, b->face_f, b->face_area, b->rctf_node,
                    b->rctf_torque, b->rctf_f, b->rctf_axis};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    free(b);
}

/* ---------------------------------------------------------------------------
 * accessors
 * ------------------------------------------------------------------------- */
int orc_blob_n_nodes(const orc_blob *b) { return b->n; }
int orc_blob_n_elem(const orc_blob *b) { return b->T; }
void orc_blob_get_pos(const orc_blob *b, double *o) { memcpy(o, b->pos, sizeof(double) * 3 * (size_t)b->n); }
void orc_blob_set_pos(orc_blob *b, const double *in) {
    memcpy(b->pos, in, sizeof(double) * 3 * (size_t)b->n);
    linearise_elements(b);
}
void orc_blob_get_vel(const orc_blob *b, double *o) { memcpy(o, b->vel, sizeof(double) * 3 * (size_t)b->n); }
void orc_blob_get_force(const orc_blob *b, double *o) { memcpy(o, b->force, sizeof(double) * 3 * (size_t)b->n); }
void orc_blob_get_rhs(const orc_blob *b, double *o) { memcpy(o, b->rhs, sizeof(double) * 3 * (size_t)b->n); }
void orc_blob_get_elem(const orc_blob *b, double *nf12, double *dpsi12, double *vol, double *vol0, double *visc144,
                       double *smag) {
    for (int e = 0; e < b->T; ++e) {
        if (nf12) memcpy(nf12 + 12 * (size_t)e, b->node_force + 30 * (size_t)e, sizeof(double) * 12);
        if (dpsi12) memcpy(dpsi12 + 12 * (size_t)e, b->dpsi + 12 * (size_t)e, sizeof(double) * 12);
    }
    if (vol) memcpy(vol, b->vol, sizeof(double) * b->T);
    if (vol0) memcpy(vol0, b->vol0, sizeof(double) * b->T);
    if (visc144) memcpy(visc144, b->visc, sizeof(double) * 144 * (size_t)b->T);
    if (smag) memcpy(smag, b->stress_mag, sizeof(double) * b->T);
}
void orc_blob_get_rest(const orc_blob *b, double *jinv9, double *mat5) {
    if (jinv9) memcpy(jinv9, b->jinv0, sizeof(double) * 9 * (size_t)b->T);
    if (mat5)
        for (int e = 0; e < b->T; ++e) {
            mat5[5 * (size_t)e] = b->rho[e]; mat5[5 * (size_t)e + 1] = b->A[e]; mat5[5 * (size_t)e + 2] = b->B[e];
            mat5[5 * (size_t)e + 3] = b->G[e]; mat5[5 * (size_t)e + 4] = b->E[e];
        }
}
double orc_blob_param(const orc_blob *b, const char *name) {
    if (!strcmp(name, "dt")) return b->dt;
    if (!strcmp(name, "kT")) return b->kT;
    if (!strcmp(name, "epsilon2")) return b->eps2;
    if (!strcmp(name, "stokes_visc")) return b->stokes_visc;
    return NAN;
}
int orc_blob_nnz(const orc_blob *b) { return b->nnz; }
void orc_blob_get_csr(const orc_blob *b, int *key, int *col, double *val, int *nsrc) {
    if (key) memcpy(key, b->key, sizeof(int) * (b->rows + 1));
    for (int k = 0; k < b->nnz; ++k) {
        if (col) col[k] = b->entry[k].col;
        if (val) val[k] = b->entry[k].val;
        if (nsrc) nsrc[k] = b->sptr[k + 1] - b->sptr[k];
    }
}
int orc_blob_n_contrib(const orc_blob *b) { return b->cptr[b->n]; }
void orc_blob_get_contrib(const orc_blob *b, int *ptr, int *es) {
    if (ptr) memcpy(ptr, b->cptr, sizeof(int) * (b->n + 1));
    if (es) memcpy(es, b->contrib_es, sizeof(int) * b->cptr[b->n]);
}
int orc_blob_mass_nnz(const orc_blob *b) { return b->mnnz; }
void orc_blob_get_mass_csr(const orc_blob *b, int *key, int *col, double *val) {
    if (key) memcpy(key, b->mkey, sizeof(int) * (b->n + 1));
    for (int k = 0; k < b->mnnz; ++k) {
        if (col) col[k] = b->mentry[k].col;
        if (val) val[k] = b->mentry[k].val;
    }
}
void orc_blob_get_inv_mass(const orc_blob *b, double *o) { if (b->inv_m) memcpy(o, b->inv_m, sizeof(double) * b->n); }
int orc_blob_last_cg_iters(const orc_blob *b) { return b->last_iters; }
long long orc_blob_total_cg_iters(const orc_blob *b) { return b->total_iters; }
void orc_blob_get_rng_state(const orc_blob *b, int t, uint32_t o[6]) { orc_rng_get_state(&b->rng[t], o); }
void orc_blob_set_rng_state(orc_blob *b, int t, const uint32_t s[6]) { orc_rng_set_state(&b->rng[t], s); }

/* Blob::make_measurements energies, src/Blob.cpp:1066-1125, of the current state: F_ij and the volume
 * are recomputed from the current positions, which is what the reference measures when it next calls
 * make_measurements (after the next update_internal_forces) */
void orc_blob_measure(const orc_blob *b, double *strain, double *kinetic) {
    double ke = 0.0, se = 0.0;
    for (int e = 0; e < b->T; ++e) {
        const int *t = b->tet + 10 * (size_t)e;
        if (b->solver != ORC_NOMASS_CG) {
            /* get_element_velocity_vector + apply_element_mass_matrix (tetra_element_linear.cpp:490-512) */
            double v[12], tmp[12] = {0};
            for (int a = 0; a < 4; ++a)
                for (int i = 0; i < 3; ++i) v[4 * i + a] = b->vel[3 * (size_t)t[a] + i];
            for (int k = 0; k < 12; k += 4)
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j) tmp[i + k] += (i == j ? .1 : .05) * v[j + k];
            for (int i = 0; i < 12; ++i) tmp[i] = tmp[i] * (b->vol0[e] * b->rho[e]);
            double s = 0;
            for (int i = 0; i < 12; ++i) s += v[i] * tmp[i];
            ke += s;
        }
        double J[3][3], F[9] = {0};
        elem_jacobian(b, e, J);
        const double c1 = J[2][2] * J[1][1] - J[2][1] * J[1][2];
        const double c2 = J[2][1] * J[0][2] - J[2][2] * J[0][1];
        const double c3 = J[1][2] * J[0][1] - J[1][1] * J[0][2];
        const double vol = (1.0 / 6.0) * fabs(J[0][0] * c1 + J[1][0] * c2 + J[2][0] * c3);
        const double *Ji = b->jinv0 + 9 * (size_t)e;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) F[3 * i + j] += J[k][i] * Ji[3 * j + k];
        const double C = b->E[e] - (2.0 / 3.0) * b->G[e];
        const double t1 = vol / b->vol0[e];
        /* mat3_double_contraction, src/mat_vec_fns.cpp:116-120 (its term order) */
        const double ff = F[0] * F[0] + F[4] * F[4] + F[8] * F[8] + F[1] * F[1] + F[3] * F[3] + F[2] * F[2] +
                          F[6] * F[6] + F[5] * F[5] + F[7] * F[7];
        se += b->vol0[e] * (b->G[e] * (ff - 3) + 0.5 * C * (t1 * t1 - 1) - (C + 2 * b->G[e]) * log(t1));
    }
    *kinetic = ke * 0.5;
    *strain = se * 0.5;
}

/* F * normalize(d) / mesoDimensions::force, as Blob::load_ctforces stores each force (src/Blob.cpp:2600-2606) */
static int ctf_convert(const double *fd, double out[3]) {
    double sum = 0; /* normalize, include/mat_vec_fns_II.h:188-198 */
    for (int i = 0; i < 3; ++i) sum += fd[1 + i] * fd[1 + i];
    if (sum == 0) return ORC_EINPUT;
    sum = sqrt(sum);
    for (int i = 0; i < 3; ++i) out[i] = fd[0] * (fd[1 + i] / sum) / MESO_FORCE;
    return ORC_OK;
}

int orc_blob_set_ctforces(orc_blob *b, int n_lin, const int *lin_node, const double *lin_fd, int n_sets,
                          const int *set_size, const int *set_faces, const double *set_fd, int n_faces,
                          const int *face_nodes) {
    int tot = 0, maxs = 0;
    for (int i = 0; i < n_lin; ++i)
        if (lin_node[i] < 0 || lin_node[i] >= b->n) return ORC_EINPUT;
    for (int s = 0; s < n_sets; ++s) {
        if (set_size[s] < 0) return ORC_EINPUT;
        tot += set_size[s];
        if (set_size[s] > maxs) maxs = set_size[s];
    }
    for (int j = 0; j < tot; ++j)
        if (set_faces[j] < 0 || set_faces[j] >= n_faces) return ORC_EINPUT;
    for (int j = 0; j < 3 * n_faces; ++j)
        if (face_nodes[j] < 0 || face_nodes[j] >= b->n) return ORC_EINPUT;
    free(b->lctf_node); free(b->lctf_f); free(b->set_size); free(b->set_faces); free(b->set_f);
    free(b->face_nodes); free(b->face_f); free(b->face_area);
    b->n_lctf = n_lin;
    b->n_sets = n_sets;
    b->n_faces = n_faces;
    b->lctf_node = xcalloc(n_lin, sizeof(int));
    b->lctf_f = xcalloc(3 * (size_t)n_lin, sizeof(double));
    b->set_size = xcalloc(n_sets, sizeof(int));
    b->set_faces = xcalloc(tot, sizeof(int));
    b->set_f = xcalloc(3 * (size_t)n_sets, sizeof(double));
    b->face_nodes = xcalloc(3 * (size_t)n_faces, sizeof(int));
    b->face_f = xcalloc(9 * (size_t)n_faces, sizeof(double));
    b->face_area = xcalloc(maxs, sizeof(double));
    for (int i = 0; i < n_lin; ++i) {
        b->lctf_node[i] = lin_node[i];
        if (ctf_convert(lin_fd + 4 * i, b->lctf_f + 3 * i)) return ORC_EINPUT;
    }
    for (int s = 0; s < n_sets; ++s) {
        b->set_size[s] = set_size[s];
        if (ctf_convert(set_fd + 4 * s, b->set_f + 3 * s)) return ORC_EINPUT;
    }
    if (tot) memcpy(b->set_faces, set_faces, sizeof(int) * tot);
    if (n_faces) memcpy(b->face_nodes, face_nodes, sizeof(int) * 3 * (size_t)n_faces);
    return ORC_OK;
}

int orc_blob_set_rot_ctforces(orc_blob *b, int n_rot, const int *rot_node, const int *rot_torque,
                              const double *rot_fpd) {
    for (int i = 0; i < n_rot; ++i)
        if (rot_node[i] < 0 || rot_node[i] >= b->n) return ORC_EINPUT;
    free(b->rctf_node); free(b->rctf_torque); free(b->rctf_f); free(b->rctf_axis);
    b->n_rctf = n_rot;
    b->rctf_node = xcalloc(n_rot, sizeof(int));
    b->rctf_torque = xcalloc(n_rot, sizeof(int));
    b->rctf_f = xcalloc(n_rot, sizeof(double));
    b->rctf_axis = xcalloc(6 * (size_t)n_rot, sizeof(double));
    for (int i = 0; i < n_rot; ++i) {
        const double *q = rot_fpd + 7 * i;
        double sum = 0; /* normalize(ctf_d), include/mat_vec_fns_II.h:188-198 */
        for (int c = 0; c < 3; ++c) sum += q[4 + c] * q[4 + c];
        if (sum == 0) return ORC_EINPUT;
        sum = sqrt(sum);
        b->rctf_node[i] = rot_node[i];
        b->rctf_torque[i] = rot_torque[i];
        b->rctf_f[i] = q[0] * (1. / MESO_FORCE); /* F * mdfm1, src/Blob.cpp:2675 */
        for (int c = 0; c < 3; ++c) {
            b->rctf_axis[6 * i + c] = (1. / MESO_LENGTH) * q[1 + c]; /* resize(mdlm1, ctf_p) */
            b->rctf_axis[6 * i + 3 + c] = q[4 + c] / sum;
        }
    }
    return ORC_OK;
}
