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

static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }
long long launch_count() { return g_launches.load(); }

cudaError_t launch_finish_step(uint32_t *rng_state, const MrgJump *step_jump, DevStatus *st, cudaStream_t s) {
    finish_step_kernel<<<1, 32, 0, s>>>(rng_state, step_jump, st);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ffea
