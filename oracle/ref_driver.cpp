/*
 * ref_driver.cpp -- drives the reference's own hot-path classes.
 *
 * TEST INFRASTRUCTURE ONLY. Built by `make ref` (oracle/Makefile) together
 * with the reference sources compiled where they lie, into _ref/libffea_ref.so.
 * It exists to pin the C restatement (orc_*.c) against the reference's real
 * code in the build container: tests/golden/gen_golden.py calls it to produce
 * the committed golden vectors.
 *
 * Only the glue that lives in Blob.cpp/World.cpp (which need Boost, Eigen
 * and program_options and are not built) is restated here, in the same
 * order as the reference; every numerical routine is the reference's:
 *   tetra_element_linear::{calculate_jacobian, calc_shape_function_derivatives_and_volume,
 *     create_viscosity_matrix, add_shear_elastic_stress, add_bulk_elastic_stress,
 *     add_fluctuating_stress, get_element_velocity_vector, apply_stress_tensor,
 *     add_element_force_vector, linearise_element, zero_force}
 *   mat3_invert, mat12_apply, mat3_double_contraction_symmetric
 *   NoMassCGSolver / ConjugateGradientSolver / MassLumpedSolver ::init / ::solve
 *   SparsityPattern, SparseMatrixFixedPattern, RngStream
 * The glue restated: Blob::init (src/Blob.cpp:161-268), load_material_params
 * (:2275-2283), calc_rest_state_info (:3080-3143),
 * calculate_node_element_connectivity (:3284-3314), update_internal_forces
 * (:400-491), aggregate_forces_and_solve (:3147-3244), linearise_force
 * (:781-799), euler_integrate (:3249-3279), make_measurements (:1066-1125).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "FFEA_return_codes.h"
#include "Face.h"
#include "RngStream.h"
#include "SimulationParams.h"
#include "Solver.h"
#include "dimensions.h"
#include "mat_vec_fns.h"
#include "mat_vec_fns_II.h"
#include "mesh_node.h"
#include "tetra_element_linear.h"
#include <omp.h>
// The solvers keep their matrices private; the driver reads them for the golden dumps.
#define private public
#include "SparseMatrixFixedPattern.h"
#include "SparsityPattern.h"
#include "ConjugateGradientSolver.h"
#include "MassLumpedSolver.h"
#include "NoMassCGSolver.h"
#undef private

// SimulationParams.cpp (script parsing, needs Boost) is not built; the two
// special members the driver needs are defined here and the hot-path fields set directly.
SimulationParams::SimulationParams() {}
SimulationParams::~SimulationParams() {}

namespace {
struct RefBlob {
    std::vector<mesh_node> node;
    std::vector<tetra_element_linear> elem;
    std::vector<arr3> force, rhs;
    std::vector<int> pinned;
    std::set<int> bsite;
    std::unique_ptr<Solver> solver;
    int solver_kind = 0;
    SimulationParams params;
    std::shared_ptr<std::vector<RngStream>> rng;
    int nthreads = 1;
    // constant forces: Blob's ctf_* members and its surface (include/Blob.h)
    std::vector<Face> surface;
    int num_l_ctf = 0, num_r_ctf = 0, num_slsets_ctf = 0;
    std::vector<int> ctf_l_nodes, ctf_r_nodes, ctf_sl_faces, ctf_sl_surfsize;
    std::vector<scalar> ctf_l_forces, ctf_r_forces, ctf_r_axis, ctf_sl_forces;
    std::vector<char> ctf_r_type;
};
}  // namespace

extern "C" {

/* RngStream passthroughs for the generator's golden vectors */
void *ref_rng_new(void) { return new RngStream(); }
void ref_rng_free(void *g) { delete static_cast<RngStream *>(g); }
int ref_rng_set_package_seed(const uint32_t s[6]) { return RngStream::SetPackageSeed(s) ? 0 : -1; }
double ref_rng_rand_u01(void *g) { return static_cast<RngStream *>(g)->RandU01(); }
int ref_rng_rand_int(void *g, int lo, int hi) { return static_cast<RngStream *>(g)->RandInt(lo, hi); }
void ref_rng_reset_start_stream(void *g) { static_cast<RngStream *>(g)->ResetStartStream(); }
void ref_rng_reset_start_substream(void *g) { static_cast<RngStream *>(g)->ResetStartSubstream(); }
void ref_rng_reset_next_substream(void *g) { static_cast<RngStream *>(g)->ResetNextSubstream(); }
void ref_rng_advance_state(void *g, int32_t e, int32_t c) { static_cast<RngStream *>(g)->AdvanceState(e, c); }
void ref_rng_set_antithetic(void *g, int a) { static_cast<RngStream *>(g)->SetAntithetic(a != 0); }
void ref_rng_increased_precis(void *g, int p) { static_cast<RngStream *>(g)->IncreasedPrecis(p != 0); }
void ref_rng_get_state(void *g, uint32_t out[6]) { static_cast<RngStream *>(g)->GetState(out); }

void *ref_blob_create(int n_nodes, const double *pos, double scale_m, int n_elem, const int *tets,
                      const double *mat6, const double *stokes_radius, int n_pinned, const int *pinned,
                      double dt, double kT, double epsilon, double stokes_visc, int max_it, int calc_noise,
                      int calc_stokes, int solver, int n_threads, int *status) {
    *status = 0;
    try {
        RefBlob *b = new RefBlob();
        SimulationParams &P = b->params;
        P.dt = dt / mesoDimensions::time;
        P.kT = kT / mesoDimensions::Energy;
        P.epsilon2 = epsilon;
        P.epsilon2 *= P.epsilon2;
        P.stokes_visc = stokes_visc / (mesoDimensions::pressure * mesoDimensions::time);
        P.max_iterations_cg = max_it;
        P.calc_noise = calc_noise;
        P.calc_stokes = calc_stokes;
        P.calc_es = 0;
        b->nthreads = n_threads;
        const scalar scale = scale_m / mesoDimensions::length;
        b->node = std::vector<mesh_node>(n_nodes);
        for (int i = 0; i < n_nodes; ++i) {
            b->node[i].pos[0] = scale * pos[3 * i];
            b->node[i].pos[1] = scale * pos[3 * i + 1];
            b->node[i].pos[2] = scale * pos[3 * i + 2];
            b->node[i].vel = {0, 0, 0};
            b->node[i].index = i;
            b->node[i].stokes_radius = stokes_radius[i] * scale;
        }
        b->elem = std::vector<tetra_element_linear>(n_elem);
        for (int e = 0; e < n_elem; ++e) {
            for (int j = 0; j < 10; ++j) b->elem[e].n[j] = &b->node[tets[10 * e + j]];
            for (int j = 0; j < 4; ++j) b->node[tets[10 * e + j]].set_linear();
            b->elem[e].index = e;
            const double *m = mat6 + 6 * e;
            b->elem[e].rho = m[0] * mesoDimensions::volume / mesoDimensions::mass;
            b->elem[e].A = m[1] / (mesoDimensions::pressure * mesoDimensions::time);
            b->elem[e].B = m[2] / (mesoDimensions::pressure * mesoDimensions::time) - (2.0 / 3.0) * m[1];
            b->elem[e].G = m[3] / mesoDimensions::pressure;
            b->elem[e].E = m[4] / mesoDimensions::pressure;
            b->elem[e].dielectric = m[5];
        }
        b->pinned.assign(pinned, pinned + n_pinned);
        for (auto &el : b->elem) el.linearise_element();
        for (auto &el : b->elem) {
            matrix3 J;
            scalar temp;
            el.calculate_jacobian(J);
            mat3_invert(J, el.J_inv_0, &temp);
            el.calc_shape_function_derivatives_and_volume(J);
            el.vol_0 = el.vol;
            el.mass = el.vol_0 * el.rho;
        }
        for (auto &nd : b->node) nd.num_element_contributors = 0;
        for (auto &el : b->elem)
            for (int j = 0; j < 10; ++j) b->node[el.n[j]->index].num_element_contributors++;
        for (auto &nd : b->node) nd.force_contributions = std::vector<arr3 *>(nd.num_element_contributors, nullptr);
        std::vector<int> counter(n_nodes, 0);
        for (auto &el : b->elem)
            for (int j = 0; j < 10; ++j) {
                const int ni = el.n[j]->index;
                b->node[ni].force_contributions[counter[ni]++] = &el.node_force[j];
            }
        b->solver_kind = solver;
        if (solver == 0) b->solver = std::make_unique<NoMassCGSolver>();
        else if (solver == 1) b->solver = std::make_unique<ConjugateGradientSolver>();
        else b->solver = std::make_unique<MassLumpedSolver>();
        b->solver->init(b->node, b->elem, P, b->pinned, b->bsite);
        b->force = std::vector<arr3>(n_nodes, {0, 0, 0});
        b->rhs = std::vector<arr3>(n_nodes, {0, 0, 0});
        if (P.calc_stokes == 1)
            for (auto &nd : b->node) nd.stokes_drag = 6.0 * ffea_const::pi * P.stokes_visc * nd.stokes_radius;
        b->rng = std::make_shared<std::vector<RngStream>>(n_threads);
        return b;
    } catch (FFEAException &) {
        *status = 3;
        return nullptr;
    }
}

void ref_blob_destroy(void *h) { delete static_cast<RefBlob *>(h); }

/* the same arguments as orc_blob_set_rot_ctforces; stored as the storing half of load_ctforces does
 * (src/Blob.cpp:2668-2730) */
int ref_blob_set_rot_ctforces(void *h, int n_rot, const int *rot_node, const int *rot_torque, const double *rot_fpd) {
    RefBlob *b = static_cast<RefBlob *>(h);
    try {
        const scalar mdfm1 = 1. / mesoDimensions::force, mdlm1 = 1. / mesoDimensions::length;
        b->num_r_ctf = n_rot;
        b->ctf_r_nodes.assign(rot_node, rot_node + n_rot);
        b->ctf_r_forces.assign(n_rot, 0.0);
        b->ctf_r_axis.assign(6 * (size_t)n_rot, 0.0);
        b->ctf_r_type.assign(2 * (size_t)n_rot, 'p');
        for (int i = 0; i < n_rot; ++i) {
            const double *q = rot_fpd + 7 * i;
            arr3 p = {q[1], q[2], q[3]}, d = {q[4], q[5], q[6]};
            normalize(d);
            resize(mdlm1, p);
            b->ctf_r_forces[i] = q[0] * mdfm1;
            for (int c = 0; c < 3; ++c) {
                b->ctf_r_axis[6 * i + c] = p[c];
                b->ctf_r_axis[6 * i + 3 + c] = d[c];
            }
            b->ctf_r_type[2 * i + 1] = rot_torque[i] ? 't' : 'f';
        }
    } catch (FFEAException &) {
        return 3;
    }
    return 0;
}

/* the same arguments as orc_blob_set_ctforces, plus the element of each face (face4: element, n0, n1, n2) */
int ref_blob_set_ctforces(void *h, int n_lin, const int *lin_node, const double *lin_fd, int n_sets,
                          const int *set_size, const int *set_faces, const double *set_fd, int n_faces,
                          const int *face4) {
    RefBlob *b = static_cast<RefBlob *>(h);
    try {
        b->surface = std::vector<Face>(n_faces);
        b->params.num_blobs = 1;
        for (int i = 0; i < n_faces; ++i) {
            const int *f = face4 + 4 * i;
            tetra_element_linear &el = b->elem[f[0]];
            const int n_op = el.get_opposite_node(el.what_node_is_this(f[1]), el.what_node_is_this(f[2]),
                                                  el.what_node_is_this(f[3]));
            if (n_op == -1) return 3;
            b->surface[i].init(i, &b->node[f[1]], &b->node[f[2]], &b->node[f[3]], el.n[n_op], nullptr, b->params);
        }
        auto conv = [](const double *fd, scalar *out) {
            arr3 d = {fd[1], fd[2], fd[3]};
            normalize(d);
            out[0] = fd[0] * d[0] / mesoDimensions::force;
            out[1] = fd[0] * d[1] / mesoDimensions::force;
            out[2] = fd[0] * d[2] / mesoDimensions::force;
        };
        b->num_l_ctf = n_lin;
        b->ctf_l_nodes.assign(lin_node, lin_node + n_lin);
        b->ctf_l_forces.assign(3 * (size_t)n_lin, 0.0);
        for (int i = 0; i < n_lin; ++i) conv(lin_fd + 4 * i, &b->ctf_l_forces[3 * i]);
        b->num_slsets_ctf = n_sets;
        b->ctf_sl_surfsize.assign(set_size, set_size + n_sets);
        int tot = 0;
        for (int s = 0; s < n_sets; ++s) tot += set_size[s];
        b->ctf_sl_faces.assign(set_faces, set_faces + tot);
        b->ctf_sl_forces.assign(3 * (size_t)n_sets, 0.0);
        for (int s = 0; s < n_sets; ++s) conv(set_fd + 4 * s, &b->ctf_sl_forces[3 * s]);
    } catch (FFEAException &) {
        return 3;
    }
    return 0;
}

/* Blob::apply_ctforces, src/Blob.cpp:1676-1741 (CTF 1 and CTF 3) */
static void apply_ctforces(RefBlob *b) {
    auto &force = b->force;
    for (int i = 0; i < b->num_l_ctf; i++) {
        force[b->ctf_l_nodes[i]][0] += b->ctf_l_forces[3 * i];
        force[b->ctf_l_nodes[i]][1] += b->ctf_l_forces[3 * i + 1];
        force[b->ctf_l_nodes[i]][2] += b->ctf_l_forces[3 * i + 2];
    }
    for (int i = 0; i < b->num_r_ctf; i++) {  // CTF 2, axes through a point ('p')
        arr3 r, f;
        mesh_node &nd = b->node[b->ctf_r_nodes[i]];
        intersectingPointToLine(nd.pos, arr_view<scalar, 3>(b->ctf_r_axis, 6 * i),
                                arr_view<scalar, 3>(b->ctf_r_axis, 6 * i + 3), r);
        sub(r, nd.pos, r);
        arr3arr3VectorProduct(r, arr_view<scalar, 3>(b->ctf_r_axis, 6 * i + 3), f);
        if (b->ctf_r_type[2 * i + 1] == 'f') {
            resize(b->ctf_r_forces[i], f);
        } else if (b->ctf_r_type[2 * i + 1] == 't') {
            const scalar rsize = magnitude(r);
            resize(b->ctf_r_forces[i] / rsize, f);
        }
        force[b->ctf_r_nodes[i]][0] += f[0];
        force[b->ctf_r_nodes[i]][1] += f[1];
        force[b->ctf_r_nodes[i]][2] += f[2];
    }
    int auxndx = 0;
    std::vector<scalar> faceAreas;
    for (int i = 0; i < b->num_slsets_ctf; i++) {
        scalar totalArea = 0;
        for (int j = 0; j < b->ctf_sl_surfsize[i]; j++) {
            faceAreas.push_back(b->surface[b->ctf_sl_faces[auxndx + j]].get_area());
            totalArea += faceAreas[j];
        }
        for (int j = 0; j < b->ctf_sl_surfsize[i]; j++) {
            arr3 traction;
            resize2(faceAreas[j] / (3 * totalArea), arr_view<scalar, 3>(b->ctf_sl_forces, 3 * i), traction);
            b->surface[b->ctf_sl_faces[auxndx + j]].add_force_to_node(0, traction);
            b->surface[b->ctf_sl_faces[auxndx + j]].add_force_to_node(1, traction);
            b->surface[b->ctf_sl_faces[auxndx + j]].add_force_to_node(2, traction);
        }
        auxndx += b->ctf_sl_surfsize[i];
        faceAreas.clear();
    }
}

static int update_internal_forces(RefBlob *b) {
    int num_inversions = 0;
    apply_ctforces(b);
    const bool nomass = b->solver_kind == 0;
#pragma omp parallel num_threads(b->nthreads) reduction(+ : num_inversions)
    {
        matrix3 J, stress;
        vector12 du;
        int tid = omp_get_thread_num();
#pragma omp for schedule(guided)
        for (int n = 0; n < (int)b->elem.size(); n++) {
            tetra_element_linear &el = b->elem[n];
            el.calculate_jacobian(J);
            if (el.calc_shape_function_derivatives_and_volume(J)) num_inversions++;
            el.create_viscosity_matrix();
            initialise(stress);
            el.add_shear_elastic_stress(J, stress);
            el.add_bulk_elastic_stress(stress);
            if (b->params.calc_noise == 1) el.add_fluctuating_stress(b->params, b->rng, stress, tid);
            el.internal_stress_mag = sqrt(mat3_double_contraction_symmetric(stress));
            if (!nomass) {
                el.get_element_velocity_vector(du);
                mat12_apply(el.viscosity_matrix, du);
            } else {
                initialise(du);
            }
            el.apply_stress_tensor(stress, du);
            el.add_element_force_vector(du);
        }
    }
    return num_inversions ? 1 : 0;
}

#define RANDH(g) ((-.5) + ((.5) - (-.5)) * ((g).RandU01()))

static int update_positions(RefBlob *b) {
    const int N = (int)b->node.size();
    const bool nomass = b->solver_kind == 0;
    auto &force = b->force;
    auto &node = b->node;
    for (int n = 0; n < N; ++n)
        for (int m = 0; m < node[n].num_element_contributors; m++) {
            force[n][0] += (*node[n].force_contributions[m])[0];
            force[n][1] += (*node[n].force_contributions[m])[1];
            force[n][2] += (*node[n].force_contributions[m])[2];
        }
    for (size_t n = 0; n < b->surface.size(); ++n)
        for (int i = 0; i < 4; i++) {
            const int sni = b->surface[n].n[i]->index;
            force[sni][0] += b->surface[n].force[i][0];
            force[sni][1] += b->surface[n].force[i][1];
            force[sni][2] += b->surface[n].force[i][2];
        }
    const SimulationParams &params = b->params;
    if (params.calc_stokes == 1 && (!nomass || params.calc_noise == 1)) {
        for (int i = 0; i < N; ++i) {
            RngStream &g = (*b->rng)[0];
            if (!nomass) {
                force[i][0] -= node[i].vel[0] * node[i].stokes_drag;
                force[i][1] -= node[i].vel[1] * node[i].stokes_drag;
                force[i][2] -= node[i].vel[2] * node[i].stokes_drag;
            }
            if (params.calc_noise == 1) {
                force[i][0] -= RANDH(g) * sqrt((24 * params.kT * node[i].stokes_drag) / (params.dt));
                force[i][1] -= RANDH(g) * sqrt((24 * params.kT * node[i].stokes_drag) / (params.dt));
                force[i][2] -= RANDH(g) * sqrt((24 * params.kT * node[i].stokes_drag) / (params.dt));
            }
        }
    }
    for (auto &el : b->elem) {
        int nIdx[10];
        for (int j = 0; j < 10; j++) nIdx[j] = el.n[j]->index;
        for (int j = 0; j < 3; j++) {
            force[nIdx[0]][j] += 0.5 * (force[nIdx[4]][j] + force[nIdx[5]][j] + force[nIdx[6]][j]);
            force[nIdx[1]][j] += 0.5 * (force[nIdx[4]][j] + force[nIdx[7]][j] + force[nIdx[8]][j]);
            force[nIdx[2]][j] += 0.5 * (force[nIdx[5]][j] + force[nIdx[7]][j] + force[nIdx[9]][j]);
            force[nIdx[3]][j] += 0.5 * (force[nIdx[6]][j] + force[nIdx[8]][j] + force[nIdx[9]][j]);
        }
        for (int j = 4; j < 10; j++) force[nIdx[j]] = {0., 0., 0.};
    }
    for (int pn : b->pinned) force[pn].fill(0);
    b->rhs = force;
    try {
        b->solver->solve(force);
    } catch (FFEAException &) {
        return 2;
    }
    for (int i = 0; i < N; ++i) {
        if (nomass) {
            for (int c = 0; c < 3; ++c) {
                node[i].vel[c] = force[i][c];
                node[i].pos[c] += force[i][c] * params.dt;
            }
        } else {
            for (int c = 0; c < 3; ++c) node[i].vel[c] += force[i][c] * params.dt;
            for (int c = 0; c < 3; ++c) node[i].pos[c] += node[i].vel[c] * params.dt;
        }
    }
    for (auto &el : b->elem) el.linearise_element();
    return 0;
}

int ref_blob_step(void *h, int nsteps) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (int s = 0; s < nsteps; ++s) {
        for (auto &el : b->elem) el.zero_force();
        for (auto &f : b->force) f = {0, 0, 0};
        for (auto &fc : b->surface) fc.zero_force();
        if (update_internal_forces(b)) return 1;
        int st = update_positions(b);
        if (st) return st;
    }
    return 0;
}

void ref_blob_get_pos(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->node.size(); ++i)
        for (int c = 0; c < 3; ++c) o[3 * i + c] = b->node[i].pos[c];
}
void ref_blob_set_pos(void *h, const double *in) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->node.size(); ++i)
        for (int c = 0; c < 3; ++c) b->node[i].pos[c] = in[3 * i + c];
    for (auto &el : b->elem) el.linearise_element();
}
void ref_blob_get_vel(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->node.size(); ++i)
        for (int c = 0; c < 3; ++c) o[3 * i + c] = b->node[i].vel[c];
}
void ref_blob_get_rhs(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->node.size(); ++i)
        for (int c = 0; c < 3; ++c) o[3 * i + c] = b->rhs[i][c];
}
void ref_blob_get_elem(void *h, double *nf12, double *dpsi12, double *vol, double *vol0, double *visc144,
                       double *smag) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t e = 0; e < b->elem.size(); ++e) {
        const tetra_element_linear &el = b->elem[e];
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 3; ++c) if (nf12) nf12[12 * e + 3 * a + c] = el.node_force[a][c];
        for (int k = 0; k < 12; ++k) if (dpsi12) dpsi12[12 * e + k] = el.dpsi[k];
        if (vol) vol[e] = el.vol;
        if (vol0) vol0[e] = el.vol_0;
        for (int r = 0; r < 12; ++r)
            for (int c = 0; c < 12; ++c) if (visc144) visc144[144 * e + 12 * r + c] = el.viscosity_matrix[r][c];
        if (smag) smag[e] = el.internal_stress_mag;
    }
}
void ref_blob_get_rest(void *h, double *jinv9, double *mat5) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t e = 0; e < b->elem.size(); ++e) {
        const tetra_element_linear &el = b->elem[e];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) if (jinv9) jinv9[9 * e + 3 * r + c] = el.J_inv_0[r][c];
        if (mat5) {
            mat5[5 * e] = el.rho; mat5[5 * e + 1] = el.A; mat5[5 * e + 2] = el.B;
            mat5[5 * e + 3] = el.G; mat5[5 * e + 4] = el.E;
        }
    }
}
int ref_blob_nnz(void *h) {
    RefBlob *b = static_cast<RefBlob *>(h);
    if (b->solver_kind != 0) return 0;
    return static_cast<NoMassCGSolver *>(b->solver.get())->V->get_num_nonzero_elements();
}
void ref_blob_get_csr(void *h, int *key, int *col, double *val, int *nsrc) {
    RefBlob *b = static_cast<RefBlob *>(h);
    auto &V = static_cast<NoMassCGSolver *>(b->solver.get())->V;
    std::vector<int> &k = V->get_key();
    std::vector<sparse_entry> &en = V->get_entries();
    if (key) std::memcpy(key, k.data(), sizeof(int) * k.size());
    for (size_t i = 0; i < en.size(); ++i) {
        if (col) col[i] = en[i].column_index;
        if (val) val[i] = en[i].val;
        if (nsrc) nsrc[i] = V->source_list[i].get_num_sources();
    }
}
int ref_blob_n_contrib(void *h) {
    RefBlob *b = static_cast<RefBlob *>(h);
    int n = 0;
    for (auto &nd : b->node) n += nd.num_element_contributors;
    return n;
}
/* contribution lists as element*10+slot, recovered from the stored pointers */
void ref_blob_get_contrib(void *h, int *ptr, int *es) {
    RefBlob *b = static_cast<RefBlob *>(h);
    const char *base = reinterpret_cast<const char *>(b->elem.data());
    int k = 0;
    ptr[0] = 0;
    for (size_t i = 0; i < b->node.size(); ++i) {
        for (arr3 *p : b->node[i].force_contributions) {
            const char *cp = reinterpret_cast<const char *>(p);
            size_t e = (size_t)(cp - base) / sizeof(tetra_element_linear);
            const char *nf0 = reinterpret_cast<const char *>(&b->elem[e].node_force[0]);
            int slot = (int)((cp - nf0) / (ptrdiff_t)sizeof(arr3));
            es[k++] = (int)(10 * e + slot);
        }
        ptr[i + 1] = k;
    }
}
int ref_blob_mass_nnz(void *h) {
    RefBlob *b = static_cast<RefBlob *>(h);
    if (b->solver_kind != 1) return 0;
    return (int)static_cast<ConjugateGradientSolver *>(b->solver.get())->entry.size();
}
void ref_blob_get_mass_csr(void *h, int *key, int *col, double *val) {
    RefBlob *b = static_cast<RefBlob *>(h);
    auto *S = static_cast<ConjugateGradientSolver *>(b->solver.get());
    std::memcpy(key, S->key.data(), sizeof(int) * S->key.size());
    for (size_t i = 0; i < S->entry.size(); ++i) {
        col[i] = S->entry[i].column_index;
        val[i] = S->entry[i].val;
    }
}
void ref_blob_get_inv_mass(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    auto *S = static_cast<MassLumpedSolver *>(b->solver.get());
    std::memcpy(o, S->inv_M.data(), sizeof(double) * S->inv_M.size());
}
void ref_blob_get_rng_state(void *h, int t, uint32_t o[6]) { (*static_cast<RefBlob *>(h)->rng)[t].GetState(o); }

void ref_blob_measure(void *h, double *strain, double *kinetic) {
    RefBlob *b = static_cast<RefBlob *>(h);
    scalar kenergy = 0.0, senergy = 0.0;
    for (auto &el : b->elem) {
        if (b->solver_kind != 0) {
            vector12 vec;
            el.get_element_velocity_vector(vec);
            el.apply_element_mass_matrix(vec);
            kenergy += el.n[0]->vel[0] * vec[0] + el.n[1]->vel[0] * vec[1] + el.n[2]->vel[0] * vec[2] +
                       el.n[3]->vel[0] * vec[3] + el.n[0]->vel[1] * vec[4] + el.n[1]->vel[1] * vec[5] +
                       el.n[2]->vel[1] * vec[6] + el.n[3]->vel[1] * vec[7] + el.n[0]->vel[2] * vec[8] +
                       el.n[1]->vel[2] * vec[9] + el.n[2]->vel[2] * vec[10] + el.n[3]->vel[2] * vec[11];
        }
        // energies of the current state: F_ij and vol from the current positions (the values the
        // reference's make_measurements sees after its next update_internal_forces)
        matrix3 J;
        el.calculate_jacobian(J);
        el.calc_deformation(J);
        el.calc_volume();
        const scalar C = el.E - (2.0 / 3.0) * el.G;
        const scalar temp1 = el.vol / el.vol_0;
        senergy += el.vol_0 * (el.G * (mat3_double_contraction(el.F_ij) - 3) + 0.5 * C * (temp1 * temp1 - 1) -
                               (C + 2 * el.G) * log(temp1));
    }
    *kinetic = kenergy * 0.5;
    *strain = senergy * 0.5;
}

}  // extern "C"
