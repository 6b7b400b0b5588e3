// engine_mixed.cu -- the mixed-precision instantiation (R = float) of the
// blob-step kernels: FP32 stress, matrix and SpMV; FP64 Jacobian inversion,
// dot-product accumulation and position accumulator.
#include "engine_impl.cuh"
#include "kernels_batch.cuh"

namespace ffea {

template struct Launch<float>;
template struct AdjLaunch<float>;

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

}  // namespace ffea
