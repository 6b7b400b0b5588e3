// engine_impl.cuh -- Launch<R> definitions; included by exactly one
// translation unit per arithmetic type (engine_fp64.cu, engine_mixed.cu).
#pragma once

#include <type_traits>

#include "engine.h"
#include "kernels_mixed.cuh"

namespace ffea {

constexpr int ELEM_THREADS = 128;
constexpr int ASM_THREADS = 128;
constexpr int GATHER_THREADS = 256;
constexpr int CG_THREADS = CG_MAX_THREADS;
constexpr int EULER_THREADS = 256;

// The FP64 element phase; the mixed path's is MixedLaunch::element (kernels_element_mixed.cuh).
template <class R>
cudaError_t Launch<R>::element(const ElemArgs<R> &a, cudaStream_t s) {
    if constexpr (std::is_same<R, float>::value) {
        return (void)a, (void)s, cudaErrorNotSupported;
    } else {
        if (a.T <= 0) return cudaSuccess;
        element_kernel<R><<<(a.T + ELEM_THREADS - 1) / ELEM_THREADS, ELEM_THREADS, 0, s>>>(a);
        count_launch();
        return cudaGetLastError();
    }
}

template <class R>
cudaError_t Launch<R>::assemble(const AsmArgs<R> &a, cudaStream_t s) {
    if (a.N <= 0 || a.nslots <= 0) return cudaSuccess;
    const int bt = a.threads > 0 ? a.threads : ASM_THREADS;
    if (!(bt == 64 || bt == 128 || bt == 256)) return cudaErrorInvalidValue;
    // by default three threads per slot while that still fits on the GPU at once (152 SMs x 2048 threads);
    // nslots is a multiple of 32, so each warp of the split kernel has one block row of 32 slots
    const bool split = a.split == 0 ? 3 * a.nslots <= 152ll * 2048 : a.split == 1;
    if (split) {
        const long long threads = 3 * a.nslots;
        assemble_kernel<R, true><<<(unsigned)((threads + bt - 1) / bt), bt, 0, s>>>(a);
    } else {
        assemble_kernel<R, false><<<(unsigned)((a.nslots + bt - 1) / bt), bt, 0, s>>>(a);
    }
    count_launch();
    return cudaGetLastError();
}

template <class R>
int Launch<R>::gather_threads() { return GATHER_THREADS; }

template <class R>
cudaError_t Launch<R>::gather(const GatherArgs<R> &a, int blocks, cudaStream_t s) {
    // modes 0 and 1 reduce over blocks of GATHER_THREADS; the batch's mode 2 takes any of 64, 128, 256
    const int bt = (a.mode == 2 && a.threads > 0) ? a.threads : GATHER_THREADS;
    if (!(bt == 64 || bt == 128 || bt == 256)) return cudaErrorInvalidValue;
    if constexpr (std::is_same<R, float>::value) {
        const bool nf = a.sn.on || a.sn.node_ctf || a.sn.vface_ptr || a.drag;
        if (a.mode == 0) {
            if (nf) gather_mixed_kernel<R, 0, true><<<blocks, bt, 0, s>>>(a);
            else gather_mixed_kernel<R, 0, false><<<blocks, bt, 0, s>>>(a);
        } else if (a.mode == 1) {
            if (nf) gather_mixed_kernel<R, 1, true><<<blocks, bt, 0, s>>>(a);
            else gather_mixed_kernel<R, 1, false><<<blocks, bt, 0, s>>>(a);
        } else {
            if (nf) gather_mixed_kernel<R, 2, true><<<blocks, bt, 0, s>>>(a);
            else gather_mixed_kernel<R, 2, false><<<blocks, bt, 0, s>>>(a);
        }
    } else {
        gather_kernel<R><<<blocks, bt, 0, s>>>(a);
    }
    count_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t Launch<R>::mid_force(const NodeForces &sn, int M, R *out, const DevStatus *st, cudaStream_t s) {
    if (M <= 0) return cudaSuccess;
    mid_force_kernel<R><<<(M + 255) / 256, 256, 0, s>>>(sn, M, out, st);
    count_launch();
    return cudaGetLastError();
}

template <class R>
int Launch<R>::cg_threads() { return CG_THREADS; }

template <class R>
int Launch<R>::cg_max_grid(int device) {
    int nsm = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    cudaError_t e;
    if constexpr (std::is_same<R, float>::value)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_mixed_kernel<R>, CG_THREADS, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_kernel<R>, CG_THREADS, 0);
    if (e != cudaSuccess) return 0;
    return nsm * per_sm;
}

// the most rows per block an owned-rows CG kernel (bytes_per_row of dynamic shared memory each) can hold
template <class K>
static int own_max_rows(K kernel, int device, int bytes_per_row) {
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return 0;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return 0;
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if (dyn <= 0 || cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
        return 0;
    const int rows = dyn / bytes_per_row;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, CG_THREADS, (size_t)rows * bytes_per_row) !=
            cudaSuccess ||
        per_sm < 1)
        return 0;
    return rows;
}

template <class R>
int Launch<R>::cg_own_max_rows(int device) {
    if constexpr (std::is_same<R, float>::value)
        return own_max_rows(cg_mixed_own_kernel<R>, device, (int)own_smem_bytes(1));
    else
        return own_max_rows(cg_own_kernel<R>, device, (int)own_smem_bytes_d(1));
}

template <class R>
int Launch<R>::cg_sr_max_rows(int device, int poly) {
    if constexpr (std::is_same<R, float>::value)
        return own_max_rows(cg_mixed_sr_kernel<R>, device, (int)sr_smem_bytes(1, poly));
    else
        return (void)device, (void)poly, 0;
}

template <class R>
int Launch<R>::cg_sr_smem_limit(int device) {
    if constexpr (std::is_same<R, float>::value) {
        int optin = 0;
        cudaFuncAttributes fa{};
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, cg_mixed_sr_kernel<R>) != cudaSuccess)
            return 0;
        const int dyn = optin - (int)fa.sharedSizeBytes;
        if (dyn <= 0 ||
            cudaFuncSetAttribute(cg_mixed_sr_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
            return 0;
        return dyn;
    } else {
        return (void)device, 0;
    }
}

template <class R>
cudaError_t Launch<R>::cg(const CgArgs<R> &a, int grid, int threads, cudaStream_t s) {
    CgArgs<R> args = a;
    void *params[] = {&args};
    const void *fn;
    size_t smem = 0;
    if constexpr (std::is_same<R, float>::value) {
        fn = (const void *)cg_mixed_kernel<R>;
        if (a.npb > 0 && a.sr) {
            fn = (const void *)cg_mixed_sr_kernel<R>;
            smem = sr_smem_bytes(a.npb, a.poly) +
                   (a.kc > 0 ? sr_cache_bytes(a.kc, sr_cache_stride(a.npb, a.tpn)) : 0);
        } else if (a.npb > 0) {
            fn = (const void *)cg_mixed_own_kernel<R>;
            smem = own_smem_bytes(a.npb);
        }
    } else {
        fn = (const void *)cg_kernel<R>;
        if (a.npb > 0) {
            fn = (const void *)cg_own_kernel<R>;
            smem = own_smem_bytes_d(a.npb);
        }
    }
    // a cooperative launch that stream capture records as a cooperative graph node
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelExC(&cfg, fn, params);
    count_launch();
    return e;
}

template <class R>
cudaError_t Launch<R>::euler(const EulerArgs<R> &a, cudaStream_t s) {
    euler_kernel<R><<<(a.N + EULER_THREADS - 1) / EULER_THREADS, EULER_THREADS, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t Launch<R>::measure(const MeasureArgs<R> &a, int blocks, double *out, cudaStream_t s) {
    measure_kernel<R><<<blocks, 256, 0, s>>>(a);
    measure_final_kernel<R><<<1, 256, 0, s>>>(a.partials, blocks, out);
    count_launch(2);
    return cudaGetLastError();
}

template <class R>
cudaError_t AdjLaunch<R>::gather(const AdjGatherArgs<R> &a, int blocks, cudaStream_t s) {
    adj_gather_kernel<R><<<blocks, 256, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t AdjLaunch<R>::modes(const AdjModesArgs &a, cudaStream_t s) {
    adj_modes_kernel<R><<<1, 256, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t AdjLaunch<R>::apply(const AdjApplyArgs<R> &a, int blocks, cudaStream_t s) {
    adj_apply_kernel<R><<<blocks, 256, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t AdjLaunch<R>::elem(const AdjElemArgs<R> &a, cudaStream_t s) {
    if (a.T <= 0) return cudaSuccess;
    elem_vjp_kernel<R><<<(a.T + 127) / 128, 128, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t AdjLaunch<R>::node(const AdjNodeArgs<R> &a, cudaStream_t s) {
    node_vjp_kernel<R><<<(a.N + 255) / 256, 256, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ffea
