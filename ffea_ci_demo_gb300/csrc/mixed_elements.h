// mixed_elements.h -- device state of the mixed-precision element phase (node_prep_kernel, element_mixed_kernel in
// kernels_element_mixed.cuh), shared by the single blob (blob.cu) and the replica batch (batch.cu).
#pragma once

#include <vector>

#include "engine.h"
#include "host_model.h"

namespace ffea {

struct MixedElements {
    double *xr = nullptr;                // 3 x N rest positions (SoA): the positions J_inv_0 was formed from
    float4 *u = nullptr, *vf = nullptr;  // FP32 displacements and (inertial solvers) velocities
    int *cta_ptr = nullptr, *cta_nodes = nullptr, *perm = nullptr, *part_ptr = nullptr;
    ushort4 *loc = nullptr;
    uint16_t *inc_local = nullptr, *inc_start = nullptr;
    float4 *parts = nullptr;             // per (block, vertex) force sums, node-major
    uint32_t *chunk_state = nullptr;     // 6 per 32-element chunk
    int *chunk_blob = nullptr, *chunk_off = nullptr;
    int N = 0, nchunks = 0;
    int threads = EM_THREADS;  // elements per thread block, as the block lists below were built
    host::Arena lists;         // the block lists and block sums (rebuilt by set_threads)

    // elem_off: first element of each blob and the total at the end (a batch), or empty (one blob, whose
    // chunk c holds elements 32c .. 32c + 31)
    cudaError_t init(host::Arena &mem, const host::HostModel &h, bool inertial, bool noise,
                     const std::vector<int> &elem_off) {
        N = h.N;
        cudaError_t e;
        if ((e = MixedLaunch::init()) != cudaSuccess) return e;
        std::vector<double> x(3 * (size_t)N);
        for (int k = 0; k < N; ++k)
            for (int c = 0; c < 3; ++c) x[(size_t)c * N + k] = h.pos[3 * (size_t)k + c];
        if ((e = mem.upload(&xr, x)) != cudaSuccess) return e;
        if ((e = mem.alloc(&u, (size_t)N)) != cudaSuccess) return e;
        if (inertial && (e = mem.alloc(&vf, (size_t)N)) != cudaSuccess) return e;
        if ((e = set_threads(h, EM_THREADS)) != cudaSuccess) return e;
        nchunks = 0;
        if (noise) {
            if (elem_off.empty()) {
                nchunks = (h.T + 31) / 32;
            } else {
                const int nb = (int)elem_off.size() - 1;
                std::vector<int> off(nb + 1, 0), cb;
                for (int b = 0; b < nb; ++b) {
                    const int nc = (elem_off[b + 1] - elem_off[b] + 31) / 32;
                    off[b + 1] = off[b] + nc;
                    cb.insert(cb.end(), nc, b);
                }
                nchunks = off[nb];
                if ((e = mem.upload(&chunk_off, off)) != cudaSuccess) return e;
                if ((e = mem.upload(&chunk_blob, cb)) != cudaSuccess) return e;
            }
            if ((e = mem.alloc(&chunk_state, 6 * (size_t)std::max(nchunks, 1))) != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    // block lists for thread blocks of t elements (64, 128 or 256); the device must be idle
    cudaError_t set_threads(const host::HostModel &h, int t) {
        if (!(t == 64 || t == 128 || t == 256)) return cudaErrorInvalidValue;
        lists.clear();
        loc = nullptr; cta_ptr = cta_nodes = perm = part_ptr = nullptr;
        inc_local = inc_start = nullptr; parts = nullptr;
        host::CtaLists cl;
        host::build_cta_lists(h, t, cl);
        std::vector<ushort4> l4(h.T);
        for (int k = 0; k < h.T; ++k)
            l4[k] = make_ushort4(cl.loc[4 * (size_t)k], cl.loc[4 * (size_t)k + 1], cl.loc[4 * (size_t)k + 2],
                                 cl.loc[4 * (size_t)k + 3]);
        cudaError_t e;
        if ((e = lists.upload(&loc, l4)) != cudaSuccess) return e;
        if ((e = lists.upload(&cta_ptr, cl.cta_ptr)) != cudaSuccess) return e;
        if ((e = lists.upload(&cta_nodes, cl.cta_nodes)) != cudaSuccess) return e;
        if ((e = lists.upload(&perm, cl.perm)) != cudaSuccess) return e;
        if ((e = lists.upload(&part_ptr, cl.part_ptr)) != cudaSuccess) return e;
        if ((e = lists.upload(&inc_local, cl.inc_local)) != cudaSuccess) return e;
        if ((e = lists.upload(&inc_start, cl.inc_start)) != cudaSuccess) return e;
        if ((e = lists.alloc(&parts, cl.cta_nodes.size())) != cudaSuccess) return e;
        threads = t;
        return cudaSuccess;
    }

    // node_prep_kernel for the state in px..vz and the streams' states (6 per blob); skip_nodes: u and vf already
    // hold the state (only the chunk states are formed)
    cudaError_t prep(const double *px, const double *py, const double *pz, const double *vx, const double *vy,
                     const double *vz, const uint32_t *rng_state, const MrgJump *chunk_jump, cudaStream_t s,
                     bool skip_nodes = false) const {
        NodePrepArgs a{};
        a.skip_nodes = skip_nodes ? 1 : 0;
        a.N = N;
        a.px = px; a.py = py; a.pz = pz; a.vx = vx; a.vy = vy; a.vz = vz;
        a.xr = xr;
        a.u = u;
        a.vf = vf;
        a.nchunks = nchunks;
        a.rng_state = rng_state;
        a.chunk_jump = chunk_jump;
        a.chunk_blob = chunk_blob;
        a.chunk_off = chunk_off;
        a.chunk_state = chunk_state;
        return MixedLaunch::node_prep(a, s);
    }

    void fill(ElemArgs<float> &ea) const {
        ea.u = u;
        ea.vf = vf;
        ea.cta_ptr = cta_ptr;
        ea.cta_nodes = cta_nodes;
        ea.loc = loc;
        ea.inc_local = inc_local;
        ea.inc_start = inc_start;
        ea.parts = parts;
        ea.perm = perm;
        ea.chunk_state = chunk_state;
        ea.chunk_off = chunk_off;
        ea.em_threads = threads;
    }
};

}  // namespace ffea
