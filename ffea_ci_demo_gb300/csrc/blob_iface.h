// blob_iface.h -- the blob handle's interface inside the library (blob.cu implements it; world.cu
// drives blobs through it). Not part of the C ABI.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/ffea_gpu.h"
#include "host_model.h"

struct ffea_gpu_adjoint {
    ffea_gpu_blob *blob;  // null once the blob is destroyed
};

struct ffea_gpu_blob {
    ffea_gpu_adjoint *adj_handle = nullptr;  // the adjoint reserved on this blob, if any
    virtual ~ffea_gpu_blob() {
        if (adj_handle) adj_handle->blob = nullptr;
    }
    ffea::host::HostModel h;
    ffea_gpu_params p{};
    uint32_t rng_host[6] = {12345, 12345, 12345, 12345, 12345, 12345};
    virtual int init() = 0;
    virtual int step(int nsteps, int *done) = 0;
    virtual int step_timed(int nsteps, long long flush_bytes, int *done, double *step_ms, double *phase_ms) = 0;
    virtual int get_state(double *pos, double *vel, double *force) = 0;
    virtual int set_state(const double *pos, const double *vel) = 0;
    virtual int set_rng(const uint32_t s[6]) = 0;
    virtual int get_rng(uint32_t s[6]) = 0;
    virtual int measure(double *se, double *ke) = 0;
    virtual int measurements(double out[6]) = 0;
    virtual int set_rmsd_reference() = 0;
    virtual int cg_iters(int *last, long long *total) = 0;
    virtual int get_elements(double *nf, double *vol, double *visc) = 0;
    virtual int get_rhs(double *rhs) = 0;
    virtual int cg_history(double *res2, int max_entries, int *count) = 0;
    virtual int cg_profile(double *ns, int n) = 0;
    virtual int cg_preconditioner(int *degree, double *lambda_max) = 0;
    virtual const char *cg_kernel_name() const = 0;
    virtual int get_matrix_values(std::vector<double> &val_sell) = 0;
    virtual int solve_static(const double *rhs, double *x, int *iterations) = 0;
    virtual int adj_init(int window, int every) = 0;
    virtual int adj_forward(int *done) = 0;
    virtual int adj_backward(const double *dl_dx, double *dG, double *dE, double *dA, double *dB,
                             double *dl_dx0) = 0;
    virtual void adj_release() = 0;
    // several blobs on one stream (the reference's single-thread order over a World's blobs): each step
    // advances the blob's stream by step_draws, and its Stokes draws start stokes_base after its elements'
    virtual int set_rng_layout(unsigned long long step_draws, unsigned long long stokes_base) = 0;
    // constant forces of the reference's ctforces file for this blob (Blob::load_ctforces)
    virtual int load_ctforces(const char *ctforces_file, const char *surface_file, int blob_index) = 0;
    // draws of one step: 7 per element (noise on) and 3 per node of the reference numbering (Stokes noise)
    unsigned long long element_draws() const { return p.calc_noise == 1 ? 7ull * (unsigned long long)h.T : 0ull; }
    unsigned long long stokes_draws() const {
        return (p.calc_noise == 1 && p.calc_stokes == 1) ? 3ull * (unsigned long long)h.n_all : 0ull;
    }
};
