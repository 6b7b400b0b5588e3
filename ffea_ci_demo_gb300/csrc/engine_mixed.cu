// engine_mixed.cu -- the mixed-precision instantiation (R = float) of the
// blob-step kernels: FP32 stress, matrix and SpMV; FP64 Jacobian inversion,
// dot-product accumulation and position accumulator.
#include "engine_impl.cuh"
#include "kernels_batch.cuh"

namespace ffea {

template struct Launch<float>;
template struct AdjLaunch<float>;

__global__ void __launch_bounds__(256) node_prep_kernel(NodePrepArgs g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.N && !g.skip_nodes) {
        const size_t N = g.N;
        g.u[i] = make_float4((float)(g.px[i] - g.xr[i]), (float)(g.py[i] - g.xr[N + i]),
                             (float)(g.pz[i] - g.xr[2 * N + i]), 0.f);
        if (g.vf) g.vf[i] = make_float4((float)g.vx[i], (float)g.vy[i], (float)g.vz[i], 0.f);
    }
    if (i < g.nchunks) {
        int b = 0, c = i;
        if (g.chunk_blob) {
            b = g.chunk_blob[i];
            c = i - g.chunk_off[b];
        }
        uint32_t s[6], o[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) s[k] = g.rng_state[6 * (size_t)b + k];
        mrg_apply(g.chunk_jump[c], s, o);
#pragma unroll
        for (int k = 0; k < 6; ++k) g.chunk_state[6 * (size_t)i + k] = o[k];
    }
}

cudaError_t MixedLaunch::node_prep(const NodePrepArgs &a, cudaStream_t s) {
    const int n = (a.N > a.nchunks && !a.skip_nodes) ? a.N : a.nchunks;
    if (n <= 0) return cudaSuccess;
    node_prep_kernel<<<(n + 255) / 256, 256, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

namespace {

template <bool PARTIALS, int NT>
cudaError_t launch_em(const ElemArgs<float> &a, int blocks, size_t smem, cudaStream_t s) {
    element_mixed_kernel<PARTIALS, NT><<<blocks, NT, smem, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <bool PARTIALS, int NT>
cudaError_t em_attribute() {
    return cudaFuncSetAttribute(element_mixed_kernel<PARTIALS, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                em_smem_bytes(NT, true, true));
}

}  // namespace

cudaError_t MixedLaunch::init() {
    // a block of 256 elements of an inertial solver with noise takes 49,664 bytes, above the default limit
    cudaError_t e;
    if ((e = em_attribute<true, 64>()) != cudaSuccess) return e;
    if ((e = em_attribute<false, 64>()) != cudaSuccess) return e;
    if ((e = em_attribute<true, 128>()) != cudaSuccess) return e;
    if ((e = em_attribute<false, 128>()) != cudaSuccess) return e;
    if ((e = em_attribute<true, 256>()) != cudaSuccess) return e;
    return em_attribute<false, 256>();
}

cudaError_t MixedLaunch::element(const ElemArgs<float> &a, bool partials, cudaStream_t s) {
    if (a.T <= 0) return cudaSuccess;
    const int nt = a.em_threads > 0 ? a.em_threads : EM_THREADS;
    const int blocks = (a.T + nt - 1) / nt;
    const size_t smem = em_smem_bytes(nt, !a.nomass, (partials || a.ef) && a.calc_noise == 1);
    switch (nt) {
    case 64:
        return partials ? launch_em<true, 64>(a, blocks, smem, s) : launch_em<false, 64>(a, blocks, smem, s);
    case 128:
        return partials ? launch_em<true, 128>(a, blocks, smem, s) : launch_em<false, 128>(a, blocks, smem, s);
    case 256:
        return partials ? launch_em<true, 256>(a, blocks, smem, s) : launch_em<false, 256>(a, blocks, smem, s);
    default:
        return cudaErrorInvalidValue;
    }
}

cudaError_t BatchLaunch::schedule(BlobCgDesc *desc, const int *blob_iters, int nblobs, int ncta, int *cta_blob,
                                  const DevStatus *st, cudaStream_t s) {
    const size_t smem = (size_t)nblobs * (2 * sizeof(double) + sizeof(int));
    schedule_kernel<<<1, 1024, smem, s>>>(desc, blob_iters, nblobs, ncta, cta_blob, st);
    count_launch();
    return cudaGetLastError();
}

cudaError_t BatchLaunch::cg(const BatchCgArgs &a, int grid, int threads, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, cg_batch_kernel, a);
    count_launch();
    return e;
}

int BatchLaunch::cg_max_grid(int device, int threads) {
    int nsm = 0, per_sm = 0;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, cg_batch_kernel) != cudaSuccess || threads > fa.maxThreadsPerBlock) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_batch_kernel, threads, 0) != cudaSuccess) return 0;
    return nsm * per_sm;
}

cudaError_t BatchLaunch::finish(uint32_t *rng_states, const MrgJump *step_jumps, int nblobs, DevStatus *st,
                                cudaStream_t s) {
    batch_finish_kernel<<<(nblobs + 127) / 128, 128, 0, s>>>(rng_states, step_jumps, nblobs, st);
    count_launch();
    return cudaGetLastError();
}

cudaError_t BatchLaunch::strain(const int4 *tet, const double *px, const double *py, const double *pz,
                                const float *jinv, const float *G, const float *E, const float *vol0, int T,
                                const int *elem_off, int nblobs, double *out, cudaStream_t s) {
    batch_strain_kernel<<<nblobs, 256, 0, s>>>(tet, px, py, pz, jinv, G, E, vol0, T, elem_off, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ffea
