// engine.h -- host-visible launchers of the blob-step kernels.
//
// The kernels are instantiated in two translation units: engine_fp64.cu
// (R = double, compiled with -fmad=false so that each FP64 expression keeps
// the reference's rounding) and engine_mixed.cu (R = float, FMA allowed).
// Host code calls them only through Launch<R>.
#pragma once

#include "batch_types.cuh"
#include "kernels_adjoint.cuh"

namespace ffea {

template <class R>
struct Launch {
    static cudaError_t element(const ElemArgs<R> &a, cudaStream_t s);
    static cudaError_t assemble(const AsmArgs<R> &a, cudaStream_t s);
    static cudaError_t gather(const GatherArgs<R> &a, int blocks, cudaStream_t s);
    // the step's midpoint forces (M midpoints) into out, for the gather's linearise replay
    static cudaError_t mid_force(const NodeForces &sn, int M, R *out, const DevStatus *st, cudaStream_t s);
    static int gather_threads();
    // persistent cooperative CG of `grid` blocks of `threads` threads (128 <= threads <= cg_threads(),
    // a multiple of 32)
    static cudaError_t cg(const CgArgs<R> &a, int grid, int threads, cudaStream_t s);
    static int cg_max_grid(int device);
    static int cg_threads();
    // mixed path: the most rows per block cg_mixed_own_kernel can keep in shared memory on `device`
    // (0: not available); a.npb > 0 selects that kernel in cg()
    static int cg_own_max_rows(int device);
    // the same for cg_mixed_sr_kernel (a.sr selects it) with a Chebyshev preconditioner of degree poly; 0 for FP64
    static int cg_sr_max_rows(int device, int poly);
    // the dynamic shared memory one cg_mixed_sr_kernel block may take on `device` (0 for FP64)
    static int cg_sr_smem_limit(int device);
    static cudaError_t euler(const EulerArgs<R> &a, cudaStream_t s);
    // measure_kernel over max(T, N, M) threads in `blocks` blocks, then the final sum into out[6]
    static cudaError_t measure(const MeasureArgs<R> &a, int blocks, double *out, cudaStream_t s);
};

// launchers of the mixed-precision element phase (kernels_element_mixed.cuh; instantiated in engine_mixed.cu)
struct MixedLaunch {
    // the element kernels' shared-memory limits on the current device; before the first launch (and outside
    // stream capture)
    static cudaError_t init();
    static cudaError_t node_prep(const NodePrepArgs &a, cudaStream_t s);
    // element_mixed_kernel over a.T elements in blocks of a.em_threads: per-block vertex sums into a.parts when
    // `partials`, else per-element forces into a.ef (when set); dpsi and volume into a.geom (when set)
    static cudaError_t element(const ElemArgs<float> &a, bool partials, cudaStream_t s);
};

// launchers of the adjoint kernels (kernels_adjoint.cuh)
template <class R>
struct AdjLaunch {
    static cudaError_t gather(const AdjGatherArgs<R> &a, int blocks, cudaStream_t s);
    static cudaError_t modes(const AdjModesArgs &a, cudaStream_t s);
    static cudaError_t apply(const AdjApplyArgs<R> &a, int blocks, cudaStream_t s);
    static cudaError_t elem(const AdjElemArgs<R> &a, cudaStream_t s);
    static cudaError_t node(const AdjNodeArgs<R> &a, cudaStream_t s);
};

extern template struct Launch<double>;
extern template struct Launch<float>;
extern template struct AdjLaunch<double>;
extern template struct AdjLaunch<float>;

cudaError_t launch_finish_step(uint32_t *rng_state, const MrgJump *step_jump, DevStatus *st, cudaStream_t s);
// the constant surface forces of a step (surf_set_kernel, then surf_face_kernel)
cudaError_t launch_surface_forces(const SurfArgs &a, cudaStream_t s);
// the step's constant node forces of the nodes with rotational forces (rot_force_kernel)
cudaError_t launch_rot_forces(const RotArgs &a, cudaStream_t s);
// node state in the reference's numbering and layout (n_all x 3, AoS) <-> the vertex rows (SoA):
// scatter takes vertex k from aos[3 node_of[k] + c]; gather writes every reference node i from its source
// rows src[i] = (a, b): a vertex (a == b), a midpoint (x_a + x_b) / 2 when `mids`, else 0 (also for a < 0)
cudaError_t launch_aos_scatter(const double *aos, const int *node_of, int N, double *px, double *py, double *pz,
                               cudaStream_t s);
cudaError_t launch_aos_gather(const double *px, const double *py, const double *pz, const int2 *src, int n_all,
                              int mids, double *aos, cudaStream_t s);

// launchers of the batch kernels (mixed precision; instantiated in engine_mixed.cu)
struct BatchLaunch {
    static cudaError_t schedule(BlobCgDesc *desc, const int *blob_iters, int nblobs, int ncta, int *cta_blob,
                                const DevStatus *st, cudaStream_t s);
    // cooperative launch of cg_batch_kernel (capturable in a CUDA graph)
    static cudaError_t cg(const BatchCgArgs &a, int grid, int threads, cudaStream_t s);
    // CTAs of `threads` threads that can be resident at once on `device`
    static int cg_max_grid(int device, int threads);
    static cudaError_t finish(uint32_t *rng_states, const MrgJump *step_jumps, int nblobs, DevStatus *st,
                              cudaStream_t s);
    // every blob's strain energy (batch_strain_kernel) into out[nblobs]
    static cudaError_t strain(const int4 *tet, const double *px, const double *py, const double *pz,
                              const float *jinv, const float *G, const float *E, const float *vol0, int T,
                              const int *elem_off, int nblobs, double *out, cudaStream_t s);
};
void count_launch(int n = 1);

}  // namespace ffea
