/*
 * ref_driver.cpp -- drives the reference's own Blob.
 *
 * TEST INFRASTRUCTURE ONLY. Built by `make ref` (oracle/Makefile) together
 * with the reference sources compiled where they lie, into _ref/libffea_ref.so.
 * It exists to pin the C restatement (orc_*.c) against the reference's real
 * code in the build container: tests/golden/gen_golden.py calls it to produce
 * the committed golden vectors.
 *
 * A blob is the reference's Blob (src/Blob.cpp), built from structure files by
 * Blob::config + Blob::init (load_nodes, load_topology, load_surface,
 * load_material_params, load_stokes_params, load_ctforces, load_pinned_nodes,
 * calc_rest_state_info, calculate_node_element_connectivity, the solver's
 * init), and stepped as World::run steps a blob (src/World.cpp:1788-2059):
 * zero_force, set_forces_to_zero, update_internal_forces (with
 * apply_ctforces), update_positions (aggregate_forces_and_solve with the
 * Stokes terms and linearise_force, the solver, euler_integrate,
 * linearise_element). Blob.cpp and its script readers compile here with the
 * test-only stand-ins in oracle/ref_shim for the Boost string helpers and the
 * Eigen types of the mode-analysis members. The only code of this file between
 * those calls: the solver Blob::init builds is wrapped so that the right-hand
 * side it is given is kept (step1_rhs), and the energies are taken from
 * Blob::make_measurements after the elements' deformation and volume are
 * brought to the current positions (tetra_element_linear's calculate_jacobian,
 * calc_deformation, calc_volume), so that they describe the current state.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "BindingSite.h"
#include "FFEA_return_codes.h"
#include "RngStream.h"
#include "SimulationParams.h"
#include "Solver.h"
#include "dimensions.h"
#include "mat_vec_fns.h"
#include "mesh_node.h"
#include "tetra_element_linear.h"
#include <omp.h>
// Blob and the solvers keep their state private; the driver reads it for the golden dumps.
#define private public
#define protected public
#include "Blob.h"
#include "ConjugateGradientSolver.h"
#include "MassLumpedSolver.h"
#include "NoMassCGSolver.h"
#include "SparseMatrixFixedPattern.h"
#include "SparsityPattern.h"
#undef private
#undef protected

namespace {
// the solver Blob::init built, keeping the right-hand side of every solve
class RecordingSolver final : public Solver {
  public:
    RecordingSolver(std::unique_ptr<Solver> s, std::vector<arr3> *rhs) : inner(std::move(s)), rhs_(rhs) {}
    void init(std::vector<mesh_node> &node, std::vector<tetra_element_linear> &elem, const SimulationParams &p,
              const std::vector<int> &pinned, const std::set<int> &bsite) override {
        inner->init(node, elem, p, pinned, bsite);
    }
    void solve(std::vector<arr3> &x) override {
        *rhs_ = x;
        inner->solve(x);
    }
    void apply_matrix(const std::vector<scalar> &in, std::vector<scalar> &result) override {
        inner->apply_matrix(in, result);
    }
    std::unique_ptr<Solver> inner;

  private:
    std::vector<arr3> *rhs_;
};

struct RefBlob {
    SimulationParams params;
    std::shared_ptr<std::vector<RngStream>> rng;
    BindingSite_matrix binding;
    Blob blob;
    Solver *inner = nullptr;
    int solver_kind = 0;  // 0 CG_nomass, 1 CG, 2 masslumped
    int nthreads = 1;     // the OpenMP threads of the Blob's parallel loops: one RngStream each
    std::vector<arr3> rhs;
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

/* Blob::config + Blob::init from structure files (ctforces may be NULL), with the hot-path keys of a script's
 * <param> block; solver 0 CG_nomass, 1 CG, 2 masslumped */
void *ref_blob_load(const char *node_file, const char *top_file, const char *surf_file, const char *mat_file,
                    const char *stokes_file, const char *pin_file, const char *ctforces_file, double scale_m, double dt,
                    double kT, double epsilon, double stokes_visc, int max_it, int calc_noise, int calc_stokes,
                    int solver, int n_threads, int *status) {
    *status = 0;
    RefBlob *b = nullptr;
    try {
        b = new RefBlob();
        SimulationParams &P = b->params;
        auto put = [&](const char *k, double v) {
            char buf[64];
            snprintf(buf, sizeof buf, "%.17g", v);
            P.assign(k, buf);
        };
        put("dt", dt);
        put("kT", kT);
        put("epsilon", epsilon);
        put("stokes_visc", stokes_visc);
        put("max_iterations_cg", max_it);
        put("calc_noise", calc_noise);
        put("calc_stokes", calc_stokes);
        P.num_blobs = 1;
        P.calc_ssint = P.calc_steric = P.calc_es = P.calc_kinetics = P.calc_preComp = P.calc_springs = 0;
        P.calc_ctforces = ctforces_file ? 1 : 0;
        if (ctforces_file) P.ctforces_fname = ctforces_file;
        b->solver_kind = solver;
        b->nthreads = n_threads;
        omp_set_num_threads(n_threads);  // Blob's loops take the default thread count (World sets it likewise)
        const int codes[3] = {FFEA_NOMASS_CG_SOLVER, FFEA_ITERATIVE_SOLVER, FFEA_MASSLUMPED_SOLVER};
        b->rng = std::make_shared<std::vector<RngStream>>(n_threads);
        // World::init's blob scale (src/World.cpp:2632): metres per file unit over the meso length
        scalar scale = scale_m;
        scale /= mesoDimensions::length;
        b->blob.config(0, 0, node_file, top_file, surf_file, mat_file, stokes_file, "", pin_file ? pin_file : "",
                       "", "", scale, 0, 1, codes[solver], FFEA_BLOB_IS_DYNAMIC, P, PreComp_params{}, nullptr,
                       &b->binding, b->rng);
        b->blob.init();
        b->inner = b->blob.solver.get();
        b->blob.solver = std::make_unique<RecordingSolver>(std::move(b->blob.solver), &b->rhs);
        b->rhs.assign(b->blob.node.size(), arr3{0, 0, 0});
        return b;
    } catch (FFEAException &) {
        delete b;
        *status = 3;
        return nullptr;
    }
}

void ref_blob_destroy(void *h) { delete static_cast<RefBlob *>(h); }

/* one World::run step of the blob (src/World.cpp:1788, 1862, 2037, 2058); 1: an element inverted (the
 * reference throws), 2: the solve failed (e.g. the CG iteration cap) */
int ref_blob_step(void *h, int nsteps) {
    RefBlob *b = static_cast<RefBlob *>(h);
    omp_set_num_threads(b->nthreads);  // as many threads as the blob has streams
    for (int s = 0; s < nsteps; ++s) {
        b->blob.zero_force();
        b->blob.set_forces_to_zero();
        try {
            b->blob.update_internal_forces();
        } catch (FFEAException &) {
            return 1;
        }
        try {
            b->blob.update_positions();
        } catch (FFEAException &) {
            return 2;
        }
    }
    return 0;
}

void ref_blob_get_pos(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->blob.node.size(); ++i)
        for (int c = 0; c < 3; ++c) o[3 * i + c] = b->blob.node[i].pos[c];
}
void ref_blob_set_pos(void *h, const double *in) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->blob.node.size(); ++i)
        for (int c = 0; c < 3; ++c) b->blob.node[i].pos[c] = in[3 * i + c];
    for (auto &el : b->blob.elem) el.linearise_element();
}
void ref_blob_get_vel(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->blob.node.size(); ++i)
        for (int c = 0; c < 3; ++c) o[3 * i + c] = b->blob.node[i].vel[c];
}
void ref_blob_get_rhs(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t i = 0; i < b->blob.node.size(); ++i)
        for (int c = 0; c < 3; ++c) o[3 * i + c] = b->rhs[i][c];
}
void ref_blob_get_elem(void *h, double *nf12, double *dpsi12, double *vol, double *vol0, double *visc144,
                       double *smag) {
    RefBlob *b = static_cast<RefBlob *>(h);
    for (size_t e = 0; e < b->blob.elem.size(); ++e) {
        const tetra_element_linear &el = b->blob.elem[e];
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
    for (size_t e = 0; e < b->blob.elem.size(); ++e) {
        const tetra_element_linear &el = b->blob.elem[e];
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
    return static_cast<NoMassCGSolver *>(b->inner)->V->get_num_nonzero_elements();
}
void ref_blob_get_csr(void *h, int *key, int *col, double *val, int *nsrc) {
    RefBlob *b = static_cast<RefBlob *>(h);
    auto &V = static_cast<NoMassCGSolver *>(b->inner)->V;
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
    for (auto &nd : b->blob.node) n += nd.num_element_contributors;
    return n;
}
/* contribution lists as element*10+slot, recovered from the stored pointers */
void ref_blob_get_contrib(void *h, int *ptr, int *es) {
    RefBlob *b = static_cast<RefBlob *>(h);
    const char *base = reinterpret_cast<const char *>(b->blob.elem.data());
    int k = 0;
    ptr[0] = 0;
    for (size_t i = 0; i < b->blob.node.size(); ++i) {
        for (arr3 *p : b->blob.node[i].force_contributions) {
            const char *cp = reinterpret_cast<const char *>(p);
            size_t e = (size_t)(cp - base) / sizeof(tetra_element_linear);
            const char *nf0 = reinterpret_cast<const char *>(&b->blob.elem[e].node_force[0]);
            int slot = (int)((cp - nf0) / (ptrdiff_t)sizeof(arr3));
            es[k++] = (int)(10 * e + slot);
        }
        ptr[i + 1] = k;
    }
}
int ref_blob_mass_nnz(void *h) {
    RefBlob *b = static_cast<RefBlob *>(h);
    if (b->solver_kind != 1) return 0;
    return (int)static_cast<ConjugateGradientSolver *>(b->inner)->entry.size();
}
void ref_blob_get_mass_csr(void *h, int *key, int *col, double *val) {
    RefBlob *b = static_cast<RefBlob *>(h);
    auto *S = static_cast<ConjugateGradientSolver *>(b->inner);
    std::memcpy(key, S->key.data(), sizeof(int) * S->key.size());
    for (size_t i = 0; i < S->entry.size(); ++i) {
        col[i] = S->entry[i].column_index;
        val[i] = S->entry[i].val;
    }
}
void ref_blob_get_inv_mass(void *h, double *o) {
    RefBlob *b = static_cast<RefBlob *>(h);
    auto *S = static_cast<MassLumpedSolver *>(b->inner);
    std::memcpy(o, S->inv_M.data(), sizeof(double) * S->inv_M.size());
}
void ref_blob_get_rng_state(void *h, int t, uint32_t o[6]) { (*static_cast<RefBlob *>(h)->rng)[t].GetState(o); }

/* Blob::make_measurements (src/Blob.cpp:1066-1125) on the current state: the elements' deformation and volume
 * are brought to the current positions first (the values its next update_internal_forces computes) */
void ref_blob_measure(void *h, double *strain, double *kinetic) {
    RefBlob *b = static_cast<RefBlob *>(h);
    omp_set_num_threads(b->nthreads);
    for (auto &el : b->blob.elem) {
        matrix3 J;
        el.calculate_jacobian(J);
        el.calc_deformation(J);
        el.calc_volume();
    }
    b->blob.make_measurements();
    *kinetic = b->blob.get_kinetic_energy();
    *strain = b->blob.get_strain_energy();
}

}  // extern "C"
