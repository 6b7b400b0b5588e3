// engine_fp64.cu -- the FP64 instantiation of the blob-step kernels.
// Compiled with -fmad=false: no multiply-add contraction, so every FP64
// expression rounds exactly as the reference's (built without FMA) does.
#include "engine_impl.cuh"

#include <atomic>

namespace ffea {

template struct Launch<double>;
template struct AdjLaunch<double>;

__global__ void finish_step_kernel(uint32_t *rng_state, const MrgJump *step_jump, DevStatus *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || st->abort) return;
    uint32_t s[6], o[6];
    for (int k = 0; k < 6; ++k) s[k] = rng_state[k];
    mrg_apply(*step_jump, s, o);
    for (int k = 0; k < 6; ++k) rng_state[k] = o[k];
    st->steps_done += 1;
}

// one thread per set: the sum of its faces' areas in file order (totalArea of apply_ctforces)
__global__ void __launch_bounds__(128) surf_set_kernel(SurfArgs g) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.nsets || g.st->abort) return;
    double total = 0.0;
    for (int k = g.set_ptr[s]; k < g.set_ptr[s + 1]; ++k) total += face_area(g, g.set_faces[k]);
    g.set_total[s] = total;
}

// one thread per face: its force from every set holding it, in set order (Face::add_force_to_node)
__global__ void __launch_bounds__(128) surf_face_kernel(SurfArgs g) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= g.nfaces || g.st->abort) return;
    double out[3] = {0.0, 0.0, 0.0};
    if (g.face_set_ptr[f] < g.face_set_ptr[f + 1]) {
        const double area = face_area(g, f);
        for (int k = g.face_set_ptr[f]; k < g.face_set_ptr[f + 1]; ++k) {
            const int s = g.face_set[k];
            const double w = area / (3 * g.set_total[s]);
            for (int c = 0; c < 3; ++c) out[c] += w * g.set_force[3 * (size_t)s + c];
        }
    }
    for (int c = 0; c < 3; ++c) g.ff[3 * (size_t)f + c] = out[c];
}

// one thread per node with rotational forces: its linear sum, then each rotational force in file order
// (Blob::apply_ctforces adds CTF 1 before CTF 2), at the node's current position (a midpoint at (x_a + x_b)/2)
__global__ void __launch_bounds__(128) rot_force_kernel(RotArgs g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nv + g.nm || g.st->abort) return;
    const bool vert = i < g.nv;
    const int j = vert ? i : i - g.nv;
    double p0[3];
    int row, e0, e1;
    const double *lin;
    double *out;
    if (vert) {
        row = g.v_row[j];
        p0[0] = g.px[row]; p0[1] = g.py[row]; p0[2] = g.pz[row];
        e0 = g.v_ptr[j]; e1 = g.v_ptr[j + 1];
        lin = g.lin_v + 3 * (size_t)row;
        out = g.out_v + 3 * (size_t)row;
    } else {
        row = g.m_idx[j];
        const int a = g.mid_a[row], b = g.mid_b[row];
        p0[0] = .5 * (g.px[a] + g.px[b]); p0[1] = .5 * (g.py[a] + g.py[b]); p0[2] = .5 * (g.pz[a] + g.pz[b]);
        e0 = g.m_ptr[j]; e1 = g.m_ptr[j + 1];
        lin = g.lin_m + 3 * (size_t)row;
        out = g.out_m + 3 * (size_t)row;
    }
    const RotEntry *ent = vert ? g.ent : g.ent_m;
    double F[3] = {lin[0], lin[1], lin[2]};
    for (int k = e0; k < e1; ++k) {
        double f[3];
        rot_force(ent[k], p0, f);
        for (int c = 0; c < 3; ++c) F[c] += f[c];
    }
    for (int c = 0; c < 3; ++c) out[c] = F[c];
}

cudaError_t launch_rot_forces(const RotArgs &a, cudaStream_t s) {
    const int n = a.nv + a.nm;
    if (n <= 0) return cudaSuccess;
    rot_force_kernel<<<(n + 127) / 128, 128, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_surface_forces(const SurfArgs &a, cudaStream_t s) {
    surf_set_kernel<<<(a.nsets + 127) / 128, 128, 0, s>>>(a);
    surf_face_kernel<<<(a.nfaces + 127) / 128, 128, 0, s>>>(a);
    count_launch(2);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) aos_scatter_kernel(const double *aos, const int *node_of, int N, double *px,
                                                          double *py, double *pz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const double *q = aos + 3 * (size_t)node_of[k];
    px[k] = q[0];
    py[k] = q[1];
    pz[k] = q[2];
}

// Blob::linearise_elements leaves every midpoint at .5 * (x_a + x_b) (tetra_element_linear::linearise_element,
// src/tetra_element_linear.cpp:553-577); a vertex is copied as is
__global__ void __launch_bounds__(256) aos_gather_kernel(const double *px, const double *py, const double *pz,
                                                         const int2 *src, int n_all, int mids, double *aos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_all) return;
    const int2 ab = src[i];
    double o0 = 0.0, o1 = 0.0, o2 = 0.0;
    if (ab.x >= 0 && ab.x == ab.y) {
        o0 = px[ab.x]; o1 = py[ab.x]; o2 = pz[ab.x];
    } else if (ab.x >= 0 && mids) {
        o0 = .5 * (px[ab.x] + px[ab.y]);
        o1 = .5 * (py[ab.x] + py[ab.y]);
        o2 = .5 * (pz[ab.x] + pz[ab.y]);
    }
    aos[3 * (size_t)i] = o0;
    aos[3 * (size_t)i + 1] = o1;
    aos[3 * (size_t)i + 2] = o2;
}

cudaError_t launch_aos_scatter(const double *aos, const int *node_of, int N, double *px, double *py, double *pz,
                               cudaStream_t s) {
    if (N <= 0) return cudaSuccess;
    aos_scatter_kernel<<<(N + 255) / 256, 256, 0, s>>>(aos, node_of, N, px, py, pz);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_aos_gather(const double *px, const double *py, const double *pz, const int2 *src, int n_all,
                              int mids, double *aos, cudaStream_t s) {
    if (n_all <= 0) return cudaSuccess;
    aos_gather_kernel<<<(n_all + 255) / 256, 256, 0, s>>>(px, py, pz, src, n_all, mids, aos);
    count_launch();
    return cudaGetLastError();
}

static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }
long long launch_count() { return g_launches.load(); }

cudaError_t launch_finish_step(uint32_t *rng_state, const MrgJump *step_jump, DevStatus *st, cudaStream_t s) {
    finish_step_kernel<<<1, 32, 0, s>>>(rng_state, step_jump, st);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ffea
