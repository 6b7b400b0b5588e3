// The adapter a maintainer adds to the reference's Blob (src/Blob.cpp) to run its per-step update on the GPU
// library (include/ffea_gpu.h). It is compiled against the reference's own headers, with these declarations
// added to class Blob (include/Blob.h:94):
//     public:  void gpu_attach(const SimulationParams &p);  void gpu_step();  void gpu_pull();
//     private: ffea_gpu_blob *gpu = nullptr;
// Like the members it replaces (Blob::update_internal_forces, update_positions) they return nothing and report a
// failure by throwing FFEAException (include/FFEA_return_codes.h:52-69).
// and World::run (src/World.cpp:1788-2059) calls gpu_step() in place of zero_force, set_forces_to_zero,
// update_internal_forces and update_positions for a blob with `gpu` set; gpu_pull() runs before
// print_trajectory_and_measurement_files, and ~Blob calls ffea_gpu_blob_destroy(gpu).
#include "Blob.h"
#include "ffea_gpu.h"

// Called once at the end of Blob::init, after calc_rest_state_info: hands the blob's structure to the GPU.
void Blob::gpu_attach(const SimulationParams &params) {
    ffea_gpu_params gp;
    ffea_gpu_params_default(&gp);
    gp.dt = params.dt; gp.kT = params.kT; gp.epsilon2 = params.epsilon2;
    gp.max_iterations_cg = params.max_iterations_cg; gp.calc_noise = params.calc_noise;
    gp.calc_stokes = params.calc_stokes; gp.stokes_visc = params.stokes_visc;
    const int ls = get_linear_solver();
    gp.solver = (ls == FFEA_NOMASS_CG_SOLVER) ? FFEA_GPU_NOMASS_CG
              : (ls == FFEA_ITERATIVE_SOLVER) ? FFEA_GPU_CG : FFEA_GPU_MASSLUMPED;
    gp.precision = FFEA_GPU_FP64;                     // or FFEA_GPU_MIXED
    std::vector<double> pos(3 * node.size()), r(node.size());
    for (size_t i = 0; i < node.size(); ++i) {
        for (int c = 0; c < 3; ++c) pos[3 * i + c] = node[i].pos[c];
        r[i] = node[i].stokes_radius;
    }
    std::vector<int> tets(10 * elem.size());
    std::vector<double> rho(elem.size()), A(elem.size()), B(elem.size()), G(elem.size()), E(elem.size());
    for (size_t e = 0; e < elem.size(); ++e) {
        for (int j = 0; j < 10; ++j) tets[10 * e + j] = elem[e].n[j]->index;
        rho[e] = elem[e].rho; A[e] = elem[e].A; B[e] = elem[e].B; G[e] = elem[e].G; E[e] = elem[e].E;
    }
    ffea_gpu_mesh m = {(int)node.size(), (int)elem.size(), (int)pinned_nodes_list.size(), pos.data(), tets.data(),
                       rho.data(), A.data(), B.data(), G.data(), E.data(), r.data(), pinned_nodes_list.data()};
    int rc = ffea_gpu_blob_create(&m, &gp, &gpu);
    if (rc) throw FFEAException("ffea_gpu_blob_create: %s", ffea_gpu_last_error());
    uint32_t s[6];
    (*rng)[0].GetState(s);                            // the blob's stream (single-thread draw order)
    if (ffea_gpu_blob_set_rng_state(gpu, s))
        throw FFEAException("ffea_gpu_blob_set_rng_state: %s", ffea_gpu_last_error());
}

// Replaces zero_force / set_forces_to_zero / update_internal_forces / update_positions for this blob.
void Blob::gpu_step() {
    int done = 0;
    switch (ffea_gpu_blob_step(gpu, 1, &done)) {
        case FFEA_GPU_OK: return;
        case FFEA_GPU_EINVERTED: throw FFEAException("Element inversion");
        case FFEA_GPU_ECGMAXIT: throw FFEAException("CG did not converge");
        default: throw FFEAException("GPU step: %s", ffea_gpu_last_error());
    }
}

// Before output (every `check` steps): copy positions and velocities back into node[] (midpoints rebuilt).
void Blob::gpu_pull() {
    std::vector<double> pos(3 * node.size()), vel(3 * node.size());
    if (ffea_gpu_blob_get_state(gpu, pos.data(), vel.data(), nullptr))
        throw FFEAException("ffea_gpu_blob_get_state: %s", ffea_gpu_last_error());
    for (size_t i = 0; i < node.size(); ++i)
        for (int c = 0; c < 3; ++c) { node[i].pos[c] = pos[3 * i + c]; node[i].vel[c] = vel[3 * i + c]; }
}
