// blob.cu -- host side of the GB300 blob-step engine and its C ABI.
//
// GpuBlob mirrors the reference's Blob (include/Blob.h:94-718) for the hot
// path: it takes the structure a Blob holds after Blob::init, keeps only the
// vertex ("linear") nodes on the device, builds the fixed 3x3-block sparsity
// pattern of the viscosity matrix once, and runs
//   element_kernel  -> update_internal_forces (src/Blob.cpp:400-491)
//   assemble_kernel -> SparseMatrixFixedPattern::build + calc_inverse_diagonal
//   gather_kernel   -> aggregate_forces_and_solve's gather (src/Blob.cpp:3147-3244)
//   cg_kernel       -> NoMassCGSolver::solve / ConjugateGradientSolver::solve
//   euler_kernel    -> euler_integrate (src/Blob.cpp:3249-3279)
// per step on one CUDA stream. Host-side arithmetic (rest state, masses,
// unit conversion) keeps the reference's evaluation order; this file is
// compiled with -ffp-contract=off on the host side.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"
#include <type_traits>

#include "engine.h"
#include "blob_iface.h"
#include "ctforces.h"
#include "ctforces_device.h"
#include "host_model.h"
#include "kernels_mixed.cuh"
#include "mixed_elements.h"

namespace ffea {
long long launch_count();
}

using namespace ffea;

using namespace ffea::host;

namespace {

// ---------------------------------------------------------------------------
// Scratch of the allocation-free solve (ffea_gpu_blob_solve_static).
//
// Some callers cannot allocate device memory at the moment they want a solve:
// a host program whose own memory pool already holds (nearly) all of the GPU's
// memory, so that a cudaMalloc would fail, or an outer integrator that calls
// the solve inside its fixed-memory time-step loop, where a cudaMalloc/cudaFree
// pair would also synchronise the whole device every call. For them the CG
// work vectors, block partial sums, grid barrier, status word and phase timers
// come from this one file-scope device array, sized for
// FFEA_GPU_SOLVE_STATIC_MAX_NODES vertex nodes (4.99 MB), instead of from the
// blob's own buffers. Each region starts on a 256-byte boundary. The array
// keeps its contents between calls: every call rewrites x, r and the partial
// sums and zeroes the status word, the barrier counters and the timers before
// the CG reads them.
// ---------------------------------------------------------------------------
constexpr int SOLVE_STATIC_MAX_NODES = FFEA_GPU_SOLVE_STATIC_MAX_NODES;
constexpr int SOLVE_PREP_THREADS = 256;
constexpr int SOLVE_MAX_BLOCKS = (SOLVE_STATIC_MAX_NODES + SOLVE_PREP_THREADS - 1) / SOLVE_PREP_THREADS;
constexpr size_t ss_round(size_t n) { return (n + 31) / 32 * 32; }  // doubles, to 256 bytes
constexpr size_t SS_VEC = 4 * (size_t)SOLVE_STATIC_MAX_NODES;        // one node vector, 4 doubles per node
constexpr size_t SS_RHS = 0;                                          // input, 3 doubles per node
constexpr size_t SS_X = SS_RHS + ss_round(3 * (size_t)SOLVE_STATIC_MAX_NODES);
constexpr size_t SS_R = SS_X + SS_VEC;
constexpr size_t SS_Q = SS_R + SS_VEC;
constexpr size_t SS_P = SS_Q + SS_VEC;
constexpr size_t SS_INIT = SS_P + SS_VEC;                             // 2 rows of SOLVE_MAX_BLOCKS
constexpr size_t SS_PART = SS_INIT + ss_round(2 * (size_t)SOLVE_MAX_BLOCKS);  // 3 rows of SOLVE_MAX_BLOCKS
constexpr size_t SS_PHASE = SS_PART + ss_round(3 * (size_t)SOLVE_MAX_BLOCKS);
constexpr size_t SS_STATUS = SS_PHASE + 32;
constexpr size_t SS_BARRIER = SS_STATUS + 32;
constexpr size_t SS_TOTAL = SS_BARRIER + 32;
static_assert(FFEA_GPU_CG_PHASES == CG_PHASES && FFEA_GPU_CG_PHASES <= 32 && sizeof(DevStatus) <= 256 && sizeof(GridBarrier) <= 256,
              "scratch regions too small");

static __device__ __align__(256) double g_solve_scratch[SS_TOTAL];

constexpr int SOLVE_STATIC_MAX_DEVICES = 64;
std::mutex g_solve_mutex;  // held for a whole call: the array is shared by every call on a device
double *g_solve_ptr[SOLVE_STATIC_MAX_DEVICES] = {};

// Device address of g_solve_scratch on `device`: looked up once per device, with that device
// current, and cached. The first lookup also loads this file's module on the device (CUDA loads
// modules lazily), which is when the array itself is placed in device memory, so blob creation
// makes this lookup for every blob that can use the allocation-free solve.
int solve_scratch(int device, double **out) {
    if (device < 0 || device >= SOLVE_STATIC_MAX_DEVICES) {
        g_last_error = "ffea_gpu_blob_solve_static: device ordinal beyond the scratch table";
        return FFEA_GPU_EINPUT;
    }
    if (!g_solve_ptr[device]) {
        int cur = -1;
        CK(cudaGetDevice(&cur));
        if (cur != device) CK(cudaSetDevice(device));
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_solve_scratch);
        if (cur != device) {
            const cudaError_t e2 = cudaSetDevice(cur);
            if (e == cudaSuccess) e = e2;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_solve_scratch)");
        g_solve_ptr[device] = static_cast<double *>(ptr);
    }
    *out = g_solve_ptr[device];
    return FFEA_GPU_OK;
}

// r = rhs, x = 0 and the block sums of |r|^2 and r.D^{-1}r that open the CG, as the gather kernel
// leaves them for a step (same per-block order, products and sums rounded separately); thread 0
// also clears the status word, the barrier counters and the phase timers.
__global__ void __launch_bounds__(SOLVE_PREP_THREADS)
    solve_static_prep_kernel(int N, const double *rhs3, const double *dinv, double *x, double *r,
                             double *init_partials, int stride, GridBarrier *gb, DevStatus *st,
                             unsigned long long *phase_ns) {
    __shared__ double smem[64];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a == 0) {
        *st = DevStatus{};
        gb->count = 0u;
        for (int k = 0; k < FFEA_GPU_CG_PHASES; ++k) phase_ns[k] = 0ull;
    }
    double acc[2] = {0.0, 0.0};
    if (a < N) {
        double F[3], z[3];
        for (int c = 0; c < 3; ++c) {
            F[c] = rhs3[3 * (size_t)a + c];
            z[c] = __dmul_rn(dinv[4 * (size_t)a + c], F[c]);
            r[4 * (size_t)a + c] = F[c];
            x[4 * (size_t)a + c] = 0.0;
        }
        acc[0] = __dadd_rn(__dadd_rn(__dmul_rn(F[0], F[0]), __dmul_rn(F[1], F[1])), __dmul_rn(F[2], F[2]));
        acc[1] = __dadd_rn(__dadd_rn(__dmul_rn(F[0], z[0]), __dmul_rn(F[1], z[1])), __dmul_rn(F[2], z[2]));
    }
    block_sum<2>(acc, smem);
    if (threadIdx.x == 0) {
        init_partials[blockIdx.x] = acc[0];
        init_partials[stride + blockIdx.x] = acc[1];
    }
}

}  // namespace

namespace {

// FP32 matrix bytes up to which the mixed CG_nomass matrix is taken to stay in the GPU's L2 (129 MB, shared with
// the vectors and the exchange buffers)
constexpr double L2_MATRIX_BYTES = 64e6;

template <class R>
struct BlobImpl final : ffea_gpu_blob {
    Arena mem;
    cudaStream_t stream = nullptr;
    int device = 0;
    // device arrays
    double *px, *py, *pz, *vx, *vy, *vz;
    int4 *tet;
    R *jinv, *G, *E, *A, *B, *vol0, *ef = nullptr, *geom = nullptr;
    double *last_det;
    int *inc_ptr, *inc, *pinned;
    int *slice_ptr, *rowlen, *bcol, *diagk, *src_ptr, *grp_slice;
    unsigned *src;
    double *drag = nullptr;
    R *val, *dinv;
    double *f;
    float *f32 = nullptr;  // mixed path: the step's assembled force, as the gather forms it (FP32)
    R *x, *r, *q, *pbuf0, *pbuf1;
    R *diag = nullptr;       // mixed path: diagonal of V
    double *partials, *init_partials;
    // the stream state. The fused mass-lumped step keeps two buffers: a step reads the current one and its gather
    // writes the next state into the other (no closing kernel), so the current buffer alternates step by step
    // (rng_cur, kept on the host; the step graphs are captured per buffer)
    uint32_t *rng_bufs[2] = {nullptr, nullptr};
    int rng_cur = 0;
    uint32_t *rng_state() const { return rng_bufs[rng_cur]; }
    MrgJump *chunk_jump, *lane_jump, *step_jump;
    DevStatus *st;
    GridBarrier *gb;
    int cg_grid = 0, gather_blocks = 0, partial_stride = 0, tpn = 4;
    int cg_npb = 0;  // rows per block of the owned-rows CG kernels (0: cg_kernel / cg_mixed_kernel)
    int cg_block = 1024;  // threads per CG block
    bool cg_sr = false;   // the mixed CG_nomass solve uses cg_mixed_sr_kernel
    int cg_poly = 0;      // with a Chebyshev preconditioner of this degree (0: Jacobi)
    int cg_kc = 0;        // and this many 3x3 blocks of each owned row in shared memory
    double *cheb = nullptr;  // its lambda_max estimate and the Lanczos record that makes it (CHEB_STATE)
    int *nb_ptr = nullptr, *nb_list = nullptr;  // its blocks' neighbour blocks
    unsigned int *nb_flags = nullptr;           // and their publication counters
    float4 *dpos = nullptr;  // mixed path: node offsets from the reference point
    MixedElements me;        // mixed path: the element phase's FP32 node data, block lists and block sums
    // measurements: densities, reference positions of vertices and midpoints (SoA), per-block sums
    R *rho = nullptr;
    double *p0 = nullptr, *m0 = nullptr, *meas_part = nullptr, *meas_out = nullptr;
    int *mid_a = nullptr, *mid_b = nullptr;
    int meas_blocks = 0;
    // constant forces (ctforces file): per vertex / midpoint linear forces, rotational forces, surface sets
    CtfDevice ctf;
    Arena lin_mem;  // the linearise replay when only the constant forces need it
    bool lin_from_ctf = false;
    // Stokes noise (calc_stokes with calc_noise)
    MrgJump *sn_chunk_jump = nullptr, *sn_lane_jump = nullptr;
    int *sn_node_orig = nullptr, *sn_mid_orig = nullptr, *sn_lin_ptr = nullptr;
    double *sn_mid_drag = nullptr;
    R *mid_f = nullptr;  // the step's midpoint forces (3 per midpoint), when any midpoint carries force
    int4 *sn_lin_ev = nullptr;
    int nmodes = 0;
    double modes[36] = {}, xc[3] = {};
    double *history = nullptr;
    unsigned long long *phase_ns = nullptr;
    int hist_cap = 0;
    cudaEvent_t ev[FFEA_GPU_NUM_PHASES + 1] = {};
    bool record_phases = false;
    // The step as a CUDA graph, replayed once per step: [0] plain, [1] with the phase events of step_timed.
    // Captured on first use. Host state that a step's launches take by value (the rigid modes and centroid,
    // constant forces, the stream layout) drops them when it changes (invalidate_graphs).
    // step graphs: [timed + 2 cont], cont = a step that follows a fused mass-lumped step of the same call (its
    // FP32 node state was written by that step's gather)
    cudaGraphExec_t gexec[8] = {};
    // graphs whose launches' by-value arguments changed (set_state's centroid and rigid modes) but not their
    // launches: re-captured on next use and updated in place, which costs less than a new instantiation
    bool refresh[8] = {};
    bool prep_cont = false;  // the step being captured is such a continuation
    // the mixed mass-lumped step with noise: the next step's chunk jumps A^(224 c + step draws), so that its gather
    // also forms the next step's chunk states and a continuation step launches no node_prep_kernel
    MrgJump *next_chunk_jump = nullptr;
    int upload_next_chunk_jumps(unsigned long long step_draws) {
        if (!next_chunk_jump) return FFEA_GPU_OK;
        const int nch = (h.T + 31) / 32;
        std::vector<MrgJump> v(nch);
        const Mat3 A224a = mat_pow(MRG_A1, 224, MRG_M1), A224b = mat_pow(MRG_A2, 224, MRG_M2);
        Mat3 ca = mat_pow(MRG_A1, step_draws, MRG_M1), cb = mat_pow(MRG_A2, step_draws, MRG_M2);
        for (int c = 0; c < nch; ++c) {
            v[c] = to_jump(ca, cb);
            ca = mat_mul(A224a, ca, MRG_M1);
            cb = mat_mul(A224b, cb, MRG_M2);
        }
        CK(cudaMemcpy(next_chunk_jump, v.data(), v.size() * sizeof(MrgJump), cudaMemcpyHostToDevice));
        return FFEA_GPU_OK;
    }
    long long graph_launches[8] = {};
    double *staging = nullptr;  // pinned host buffer, 3*N doubles, for state copies
    // node state in the reference's layout on the device: n_all x 3 doubles, the vertex row of each vertex
    // node, and the source rows of every reference node (vertex (k, k), midpoint (a, b), else (-1, -1))
    double *aos = nullptr;
    int *d_node_of = nullptr;
    int2 *ref_src = nullptr;
    // adjoint window (ffea_gpu_adjoint_*): checkpoints every `adj_every` steps, one segment recomputed
    std::unique_ptr<Arena> adj_mem;
    int adj_window = 0, adj_every = 0, adj_done = -1;
    double *ck_pos = nullptr, *ck_det = nullptr, *seg_pos = nullptr, *lam = nullptr, *eg = nullptr,
           *gtheta = nullptr, *coef = nullptr, *adj_part_d = nullptr, *fin_pos = nullptr, *fin_det = nullptr;
    uint32_t *ck_rng = nullptr, *seg_rng = nullptr, *fin_rng = nullptr;
    R *seg_v = nullptr;
    float2 *adj_part_f = nullptr;

    ~BlobImpl() override {
        invalidate_graphs();
        if (staging) cudaFreeHost(staging);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }

    int mark(int k) {
        // an event record node when the step is being captured
        if (record_phases) CK(cudaEventRecordWithFlags(ev[k], stream, cudaEventRecordExternal));
        return FFEA_GPU_OK;
    }

    void invalidate_graphs() {
        for (auto &g : gexec)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
        for (auto &r : refresh) r = false;
    }

    // the mixed mass-lumped step leaves the next step's FP32 node state behind (its gather updates the positions)
    bool fused_prep() const { return std::is_same<R, float>::value && p.solver == FFEA_GPU_MASSLUMPED; }

    // one step through its graph (captured from launch_step on first use); `cont`: the previous launch on the
    // stream was a step of the same call, so a fused step need not form the FP32 node state again
    int launch_step_graph(int timed, bool cont = false) {
        const int gi = timed + ((cont && fused_prep()) ? 2 : 0) + 4 * rng_cur;
        if (!gexec[gi] || refresh[gi]) {
            record_phases = timed != 0;
            prep_cont = (gi & 2) != 0;
            const long long l0 = launch_count();
            CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            const int rc = launch_step();
            cudaGraph_t graph = nullptr;
            const cudaError_t e = cudaStreamEndCapture(stream, &graph);
            record_phases = false;
            prep_cont = false;
            graph_launches[gi] = launch_count() - l0;
            count_launch((int)-graph_launches[gi]);  // counted on every replay instead
            if (rc || e != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return rc ? rc : cuda_fail(e, "cudaStreamEndCapture");
            }
            refresh[gi] = false;
            if (gexec[gi]) {
                // the same launches with new arguments: update the instantiated graph; if the update is refused,
                // instantiate anew (the refusal is not a sticky error, but it is cleared from the last-error slot)
                cudaGraphExecUpdateResultInfo info{};
                if (cudaGraphExecUpdate(gexec[gi], graph, &info) != cudaSuccess) {
                    (void)cudaGetLastError();
                    cudaGraphExecDestroy(gexec[gi]);
                    gexec[gi] = nullptr;
                }
            }
            cudaError_t ei = cudaSuccess;
            if (!gexec[gi]) ei = cudaGraphInstantiate(&gexec[gi], graph, 0);
            cudaGraphDestroy(graph);
            if (ei != cudaSuccess) {
                gexec[gi] = nullptr;
                return cuda_fail(ei, "cudaGraphInstantiate");
            }
        }
        CK(cudaGraphLaunch(gexec[gi], stream));
        count_launch((int)graph_launches[gi]);
        return FFEA_GPU_OK;
    }

    int init() override {
        CK(cudaGetDevice(&device));
        int major = 0, minor = 0;
        CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
        CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
        if (major != 10 || minor != 3) {
            g_last_error = "this library is built for sm_103a (GB300) only";
            return FFEA_GPU_ECUDA;
        }
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        for (auto &e : ev) CK(cudaEventCreate(&e));
        CK(cudaHostAlloc((void **)&staging, 3 * (size_t)std::max(h.N, 1) * sizeof(double), cudaHostAllocDefault));
        const int N = h.N, T = h.T;
        std::vector<double> tmp(N);
        auto up3 = [&](double **dst, int c) -> cudaError_t {
            for (int k = 0; k < N; ++k) tmp[k] = h.pos[3 * (size_t)k + c];
            return mem.upload(dst, tmp);
        };
        CK(up3(&px, 0));
        CK(up3(&py, 1));
        CK(up3(&pz, 2));
        {
            std::vector<int2> src(std::max(h.n_all, 1), make_int2(-1, -1));
            for (int k = 0; k < N; ++k) src[h.node_of[k]] = make_int2(k, k);
            for (size_t m = 0; m < h.mid_nodes.size(); ++m) src[h.mid_nodes[m]] = make_int2(h.mid_a[m], h.mid_b[m]);
            CK(mem.upload(&ref_src, src));
            CK(mem.upload(&d_node_of, h.node_of));
            CK(mem.alloc(&aos, 3 * (size_t)std::max(h.n_all, 1)));
        }
        CK(mem.alloc(&vx, N));
        CK(mem.alloc(&vy, N));
        CK(mem.alloc(&vz, N));
        std::vector<int4> t4(T);
        for (int e = 0; e < T; ++e)
            t4[e] = make_int4(h.tet4[4 * (size_t)e], h.tet4[4 * (size_t)e + 1], h.tet4[4 * (size_t)e + 2],
                              h.tet4[4 * (size_t)e + 3]);
        CK(mem.upload(&tet, t4));
        std::vector<R> js(9 * (size_t)T);
        for (int e = 0; e < T; ++e)
            for (int k = 0; k < 9; ++k) js[(size_t)k * T + e] = (R)h.jinv[9 * (size_t)e + k];
        CK(mem.upload(&jinv, js));
        CK(mem.upload(&G, cast_vec<R>(h.G)));
        CK(mem.upload(&E, cast_vec<R>(h.E)));
        CK(mem.upload(&A, cast_vec<R>(h.A)));
        CK(mem.upload(&B, cast_vec<R>(h.B)));
        CK(mem.upload(&vol0, cast_vec<R>(h.vol0)));
        CK(mem.upload(&rho, cast_vec<R>(h.rho)));
        {
            const int M = (int)h.mid_nodes.size();
            std::vector<double> q0(3 * (size_t)N), qm(3 * (size_t)std::max(M, 1));
            for (int k = 0; k < N; ++k)
                for (int c = 0; c < 3; ++c) q0[(size_t)c * N + k] = h.pos[3 * (size_t)k + c];
            for (int m = 0; m < M; ++m)
                for (int c = 0; c < 3; ++c)
                    qm[(size_t)c * M + m] = .5 * (h.pos[3 * (size_t)h.mid_a[m] + c] + h.pos[3 * (size_t)h.mid_b[m] + c]);
            CK(mem.upload(&p0, q0));
            CK(mem.upload(&m0, qm));
            CK(mem.upload(&mid_a, h.mid_a));
            CK(mem.upload(&mid_b, h.mid_b));
            meas_blocks = (std::max({T, N, M}) + 255) / 256;
            CK(mem.alloc(&meas_part, (size_t)MEASURE_NV * meas_blocks));
            CK(mem.alloc(&meas_out, (size_t)MEASURE_NV));
        }
        CK(mem.upload(&last_det, h.last_det));
        // element forces and geometry per element: the FP64 path keeps both (the gather reads the forces in the
        // reference's order); the mixed path sums forces per thread block and keeps geometry for the assembly only
        if (!std::is_same<R, float>::value) CK(mem.alloc(&ef, 12 * (size_t)T));
        if (!std::is_same<R, float>::value || p.solver == FFEA_GPU_NOMASS_CG) CK(mem.alloc(&geom, 16 * (size_t)T));
        CK(mem.upload(&inc_ptr, h.inc_ptr));
        CK(mem.upload(&inc, h.inc));
        CK(mem.upload(&pinned, h.pinned));
        CK(mem.upload(&slice_ptr, h.slice_ptr));
        CK(mem.upload(&rowlen, h.rowlen));
        CK(mem.upload(&bcol, h.bcol));
        CK(mem.upload(&diagk, h.diagk));
        CK(mem.upload(&grp_slice, h.grp_slice));
        CK(mem.upload(&src_ptr, h.src_ptr));
        CK(mem.upload(&src, h.src));
        if (!h.drag.empty()) CK(mem.upload(&drag, h.drag));
        const bool block3 = p.solver == FFEA_GPU_NOMASS_CG;
        if (p.solver == FFEA_GPU_CG) {
            CK(mem.upload(&val, cast_vec<R>(h.mass_sell)));
        } else {
            CK(mem.alloc(&val, (block3 ? 9 : 1) * (size_t)h.nslots));
        }
        // Jacobi preconditioner (CG solver: 1/diag of the constant mass matrix) or lumped inverse mass
        std::vector<R> dv(4 * (size_t)N, (R)0);
        if (p.solver == FFEA_GPU_CG) {
            for (int a = 0; a < N; ++a) {
                const int s = a >> 5, lane = a & 31;
                const double d = h.mass_sell[h.slice_ptr[s] + 32 * h.diagk[a] + lane];
                for (int c = 0; c < 3; ++c) dv[4 * (size_t)a + c] = (R)(1.0 / d);
            }
        } else if (p.solver == FFEA_GPU_MASSLUMPED) {
            for (int a = 0; a < N; ++a)
                for (int c = 0; c < 3; ++c) dv[4 * (size_t)a + c] = (R)h.inv_mass[a];
        }
        CK(mem.upload(&dinv, dv));
        CK(mem.alloc(&f, 4 * (size_t)N));
        if (std::is_same<R, float>::value) CK(mem.alloc(&f32, 4 * (size_t)N));
        CK(mem.alloc(&x, 4 * (size_t)N));
        CK(mem.alloc(&r, 4 * (size_t)N));
        CK(mem.alloc(&pbuf0, 4 * (size_t)N));
        CK(mem.alloc(&pbuf1, 4 * (size_t)N));
        CK(mem.alloc(&q, 4 * (size_t)N));
        const int gthreads = Launch<R>::gather_threads();
        gather_blocks = (N + gthreads - 1) / gthreads;
        constexpr bool mixed = std::is_same<R, float>::value;
        CK(mem.alloc(&init_partials, (mixed ? MIXED_GATHER_NP : 2) * (size_t)gather_blocks));
        if (mixed) {
            CK(mem.alloc(&diag, 4 * (size_t)N));
            CK(mem.alloc(&dpos, (size_t)N));
            CK(me.init(mem, h, p.solver != FFEA_GPU_NOMASS_CG, p.calc_noise == 1, {}));
        }
        // rigid modes: the mixed CG deflates them; both paths' adjoints project them out
        nmodes = rigid_modes(h, p, xc, modes);
        const int maxg = Launch<R>::cg_max_grid(device);
        if (maxg <= 0) {
            g_last_error = "cg kernel cannot be made resident";
            return FFEA_GPU_ECUDA;
        }
        // one block per SM (fewer for small meshes). A mixed blob of up to 2048 rows runs in a single block (its
        // barrier is a block barrier); an FP64 one only up to 256 rows, since its SpMV is bound by the FP64
        // units of the SMs it runs on. A single block has as few threads as give each row 8 lanes. Threads per
        // SpMV row chosen so that every warp handles its rows in one pass: tpn = the largest power of two <= 8
        // with N <= warps * 32 / tpn
        if (N <= (mixed ? 2048 : 256)) {
            cg_grid = 1;
            cg_block = std::min(Launch<R>::cg_threads(), std::max(128, (N * 8 + 31) / 32 * 32));
        } else {
            cg_grid = std::max(1, std::min(maxg, (N + 255) / 256));
            cg_block = Launch<R>::cg_threads();
        }
        const long long lanes = (long long)cg_grid * cg_block;
        tpn = 8;
        while (tpn > 1 && (long long)N * tpn > lanes) tpn >>= 1;
        partial_stride = cg_grid;
        // The CG kernel follows from the blob's size alone (no other input selects it):
        //  - each block keeps a run of rows in shared memory when they fit (cg_own_kernel, cg_mixed_own_kernel);
        //    the run is a multiple of a warp's rows so that a warp's rows share a SELL slice; else the grid-strided
        //    cg_kernel / cg_mixed_kernel;
        //  - the mixed CG_nomass solve takes one reduction per iteration (cg_mixed_sr_kernel) when its rows fit and
        //    its FP32 matrix stays in L2
        {
            const int maxrows = Launch<R>::cg_own_max_rows(device);
            const int align = 32 / tpn, rows = (N + cg_grid - 1) / cg_grid;
            const int npb = (rows + align - 1) / align * align;
            cg_npb = (maxrows > 0 && npb <= maxrows) ? npb : 0;
            // ... while its FP32 matrix (40 B per 3x3 block) stays in L2: once the SpMV streams the matrix from HBM
            // the two-reduction kernel's iterations are the shorter ones (64^3 cells: 38.7 against 43.5 us)
            const bool l2_resident = 40.0 * (double)h.nslots <= L2_MATRIX_BYTES;
            if (mixed && p.solver == FFEA_GPU_NOMASS_CG && maxrows > 0 && l2_resident) {
                // the polynomial preconditioner's two extra vectors per row must fit as well; else Jacobi
                const int poly = p.cg_poly == 0 ? FFEA_GPU_CG_POLY_DEFAULT : std::max(p.cg_poly, 0);
                for (int deg : {poly, 0}) {
                    const int srrows = Launch<R>::cg_sr_max_rows(device, deg);
                    if (srrows > 0 && npb <= srrows) {
                        cg_sr = true;
                        cg_poly = deg;
                        break;
                    }
                }
                if (cg_sr) cg_npb = npb;
            }
            if (cg_sr) {
                // the first blocks of each owned row kept in shared memory for the solve, as many as the rest of
                // the block's shared memory holds (ffea_gpu_params::cg_smem_blocks caps them: n > 0 at most n, -1
                // none; the results do not depend on it)
                // The block's shared memory stops at 168 KB so that L1 (the rest of the SM's 256 KB) keeps the
                // neighbours' exchanged vectors: on the 40^3 cube 6 cached blocks per row (167 KB) gave 20.8 us per
                // iteration, the 9 that fit (223 KB) 21.4 us, none 22.3 us.
                const long long avail = std::min<long long>(Launch<R>::cg_sr_smem_limit(device), 168 * 1024) -
                                        (long long)sr_smem_bytes(cg_npb, cg_poly);
                const long long S = sr_cache_stride(cg_npb, tpn);
                int maxlen = 0;
                for (int a = 0; a < N; ++a) maxlen = std::max(maxlen, h.rowlen[a]);
                cg_kc = avail <= 0 ? 0 : (int)std::min<long long>(maxlen, avail / (SR_CACHE_BYTES_PER_BLOCK * S));
                if (p.cg_smem_blocks != 0) cg_kc = std::min(cg_kc, std::max(0, p.cg_smem_blocks));
            }
            if (cg_poly > 0) {
                CK(mem.alloc(&cheb, (size_t)CHEB_STATE));
                CK(cudaMemset(cheb, 0, CHEB_STATE * sizeof(double)));
            }
            // the FP64 owned-rows CG publishes its search direction the same way (CG_nomass's 3x3 pattern)
            if (cg_sr || (!mixed && cg_npb > 0 && p.solver == FFEA_GPU_NOMASS_CG)) {
                // the blocks each block's SpMV reads z (p) from: owners of the columns of its rows. The pattern is
                // symmetric (an element couples each pair of its unpinned nodes both ways; a pinned row keeps only
                // its diagonal and no row has its column), so these are also the blocks that read from it, which
                // the exchange's buffer reuse relies on.
                std::vector<int> nbp(cg_grid + 1, 0), nbl;
                std::vector<char> seen(cg_grid, 0);
                for (int b = 0; b < cg_grid; ++b) {
                    std::vector<int> got;
                    for (int a = b * npb; a < std::min(N, (b + 1) * npb); ++a) {
                        const int s0 = h.slice_ptr[a >> 5], ln = a & 31;
                        for (int k = 0; k < h.rowlen[a]; ++k) {
                            const int ob = h.bcol[s0 + 32 * k + ln] / npb;
                            if (ob != b && !seen[ob]) { seen[ob] = 1; got.push_back(ob); }
                        }
                    }
                    for (int ob : got) seen[ob] = 0;
                    std::sort(got.begin(), got.end());
                    nbl.insert(nbl.end(), got.begin(), got.end());
                    nbp[b + 1] = (int)nbl.size();
                }
                if (nbl.empty()) nbl.push_back(0);
                CK(mem.upload(&nb_ptr, nbp));
                CK(mem.upload(&nb_list, nbl));
                CK(mem.alloc(&nb_flags, (size_t)FLAG_STRIDE * cg_grid));
            }
        }
        CK(mem.alloc(&partials, (mixed ? std::max(MIXED_PARTIAL_ROWS, MIXED_SR_NP) : 3) * (size_t)partial_stride));
        CK(mem.alloc(&st, 1));
        hist_cap = std::min(std::max(p.max_iterations_cg, 1), 1 << 20);
        CK(mem.alloc(&history, (size_t)hist_cap));
        CK(mem.alloc(&phase_ns, (size_t)FFEA_GPU_CG_PHASES));
        CK(mem.alloc(&gb, 1));
        // RNG jump tables: draws of element e start 7e after the step's state; a step consumes 7T
        const int nchunks = (T + 31) / 32;
        std::vector<MrgJump> cj(nchunks), lj(32);
        const Mat3 A224a = mat_pow(MRG_A1, 224, MRG_M1), A224b = mat_pow(MRG_A2, 224, MRG_M2);
        Mat3 ca{}, cb{};
        for (int i = 0; i < 3; ++i) ca.m[i][i] = cb.m[i][i] = 1;
        for (int c = 0; c < nchunks; ++c) {
            cj[c] = to_jump(ca, cb);
            ca = mat_mul(A224a, ca, MRG_M1);
            cb = mat_mul(A224b, cb, MRG_M2);
        }
        for (int l = 0; l < 32; ++l) lj[l] = jump_pow(7ull * l);
        CK(mem.upload(&chunk_jump, cj));
        CK(mem.upload(&lane_jump, lj));
        // a step consumes 7 draws per element when noise is on (and 3 per node of the reference numbering
        // with Stokes drag), none otherwise
        const bool snoise = p.calc_noise == 1 && p.calc_stokes == 1;
        CK(mem.alloc(&step_jump, 1));
        if (snoise) {
            CK(mem.alloc(&sn_chunk_jump, (size_t)(h.n_all + 31) / 32));
            std::vector<MrgJump> nlj(32);
            for (int l = 0; l < 32; ++l) nlj[l] = jump_pow(3ull * l);
            CK(mem.upload(&sn_lane_jump, nlj));
            CK(mem.upload(&sn_node_orig, h.node_of));
            std::vector<double> mdrag(h.mid_nodes.size());
            for (size_t m = 0; m < h.mid_nodes.size(); ++m) mdrag[m] = h.drag_all[h.mid_nodes[m]];
            CK(mem.upload(&sn_mid_orig, h.mid_nodes));
            CK(mem.upload(&sn_mid_drag, mdrag));
            if (!h.mid_nodes.empty()) CK(mem.alloc(&mid_f, 3 * h.mid_nodes.size()));
            int lrc0 = upload_linearise(mem);
            if (lrc0) return lrc0;
        }
        if (fused_prep() && p.calc_noise == 1) CK(mem.alloc(&next_chunk_jump, (size_t)nchunks));
        int lrc = set_rng_layout(element_draws() + stokes_draws(), element_draws());
        if (lrc) return lrc;
        std::vector<uint32_t> rs(rng_host, rng_host + 6);
        CK(mem.upload(&rng_bufs[0], rs));
        if (fused_prep()) CK(mem.alloc(&rng_bufs[1], 6));
        // a blob that the allocation-free solve accepts gets the static scratch placed now, and that solve's
        // kernels loaded (cg_kernel by the occupancy query above), so that its first solve allocates nothing
        if (!mixed && p.solver != FFEA_GPU_MASSLUMPED && N <= SOLVE_STATIC_MAX_NODES && cg_grid <= SOLVE_MAX_BLOCKS) {
            double *ss = nullptr;
            const int src = solve_scratch(device, &ss);
            if (src) return src;
            cudaFuncAttributes fa{};
            CK(cudaFuncGetAttributes(&fa, solve_static_prep_kernel));
        }
        CK(cudaDeviceSynchronize());
        return FFEA_GPU_OK;
    }

    ElemArgs<R> elem_args(int recompute) {
        ElemArgs<R> ea{};
        ea.T = h.T;
        ea.nomass = p.solver == FFEA_GPU_NOMASS_CG;
        ea.calc_noise = p.calc_noise;
        ea.kT = (R)p.kT;
        ea.dt = (R)p.dt;
        ea.tet = tet;
        ea.px = px; ea.py = py; ea.pz = pz;
        ea.vx = vx; ea.vy = vy; ea.vz = vz;
        ea.jinv = jinv;
        ea.G = G; ea.E = E; ea.A = A; ea.B = B; ea.vol0 = vol0;
        ea.last_det = last_det;
        ea.ef = ef;
        ea.geom = geom;
        ea.rng_state = rng_state();
        ea.chunk_jump = chunk_jump;
        ea.lane_jump = lane_jump;
        ea.recompute = recompute;
        ea.st = st;
        return ea;
    }

    // the element phase: FP64 element_kernel, or (mixed) node_prep_kernel and element_mixed_kernel, which sums
    // each thread block's forces per vertex for the gather; `recompute` (the adjoint's re-evaluation at stored
    // positions) needs only the geometry the assembly reads
    int launch_elements(int recompute) {
        if constexpr (std::is_same<R, float>::value) {
            // a continuation step of the fused mass-lumped path finds its node state and chunk states ready
            const bool cont = prep_cont && !recompute;
            if (!cont || (me.nchunks > 0 && !next_chunk_jump))
                CK(me.prep(px, py, pz, vx, vy, vz, rng_state(), chunk_jump, stream, cont));
            ElemArgs<float> ea = elem_args(recompute);
            me.fill(ea);
            ea.ef = nullptr;
            ea.geom = p.solver == FFEA_GPU_NOMASS_CG ? geom : nullptr;
            if (recompute) ea.parts = nullptr;
            CK(MixedLaunch::element(ea, !recompute, stream));
        } else {
            CK(Launch<R>::element(elem_args(recompute), stream));
        }
        return FFEA_GPU_OK;
    }

    int launch_assemble() {
        AsmArgs<R> aa{};
        aa.N = h.N;
        aa.nslots = h.nslots; aa.grp_slice = grp_slice;
        aa.slice_ptr = slice_ptr; aa.rowlen = rowlen; aa.bcol = bcol; aa.diagk = diagk;
        aa.src_ptr = src_ptr; aa.src = src;
        aa.geom = geom; aa.A = A; aa.B = B;
        aa.drag = (p.calc_stokes == 1) ? drag : nullptr;
        aa.val = val; aa.dinv = dinv; aa.diag = diag; aa.st = st;
        CK(Launch<R>::assemble(aa, stream));
        return FFEA_GPU_OK;
    }

    // the CG of a step, opened by the gather's (or the adjoint gather's) block sums in `init`
    int launch_cg(const double *init, int n_init) {
        const bool nomass = p.solver == FFEA_GPU_NOMASS_CG;
        CgArgs<R> ca{};
        ca.N = h.N;
        ca.block3 = nomass;
        ca.check_last = nomass;
        ca.slice_ptr = slice_ptr; ca.rowlen = rowlen; ca.bcol = bcol;
        ca.val = val; ca.dinv = dinv;
        ca.x = x; ca.r = r; ca.q = q; ca.pbuf0 = pbuf0; ca.pbuf1 = pbuf1; ca.diag = diag;
        ca.init_partials = init; ca.n_init = n_init; ca.init_stride = gather_blocks;
        ca.partials = partials; ca.stride = partial_stride;
        ca.gb = gb; ca.st = st;
        ca.imax = p.max_iterations_cg;
        ca.eps2 = p.epsilon2;
        ca.limit_ns = 2000000000ull;
        ca.history = history; ca.hist_cap = hist_cap; ca.tpn = tpn; ca.phase_ns = phase_ns;
        CK(cudaMemsetAsync(phase_ns, 0, FFEA_GPU_CG_PHASES * sizeof(unsigned long long), stream));
        ca.dpos = dpos; ca.nmodes = nomass ? nmodes : 0;
        for (int i = 0; i < 36; ++i) ca.modes[i] = modes[i];
        ca.npb = cg_npb;
        ca.sr = cg_sr && nomass;
        ca.poly = ca.sr ? cg_poly : 0;
        ca.kc = ca.sr ? cg_kc : 0;
        ca.cheb = cheb;
        // a Chebyshev step (SpMV + neighbour exchange) against a whole iteration (SpMV, exchange, grid-wide
        // reduction): about half while the FP32 matrix (40 B per 3x3 block) stays in L2, more once it streams
        // from HBM
        ca.cheb_cost = 40.0 * (double)h.nslots <= L2_MATRIX_BYTES ? 0.5f : 0.9f;
        if (nb_flags) {
            ca.nb_ptr = nb_ptr; ca.nb_list = nb_list; ca.flags = nb_flags;
            CK(cudaMemsetAsync(nb_flags, 0, (size_t)FLAG_STRIDE * cg_grid * sizeof(unsigned int), stream));
        }
        CK(Launch<R>::cg(ca, cg_grid, cg_block, stream));
        return FFEA_GPU_OK;
    }

    int launch_step() {
        const bool nomass = p.solver == FFEA_GPU_NOMASS_CG;
        int rc = mark(0);
        if (rc) return rc;
        if ((rc = launch_elements(0))) return rc;
        if ((rc = mark(1))) return rc;
        if (nomass && (rc = launch_assemble())) return rc;
        if ((rc = mark(2))) return rc;
        GatherArgs<R> ga{};
        ga.N = h.N;
        ga.mode = p.solver == FFEA_GPU_MASSLUMPED ? 1 : 0;
        ga.inc_ptr = inc_ptr; ga.inc = inc; ga.ef = ef; ga.pinned = pinned;
        ga.parts = me.parts; ga.part_ptr = me.part_ptr;
        ga.drag = (!nomass && p.calc_stokes == 1) ? drag : nullptr;
        ga.vx = vx; ga.vy = vy; ga.vz = vz;
        ga.dinv = dinv; ga.x = x; ga.r = r;
        if (f32) ga.f32 = f32; else ga.f = f;
        ga.partials = init_partials; ga.stride = gather_blocks; ga.st = st; ga.gb = gb;
        ga.dpos = dpos; ga.px = px; ga.py = py; ga.pz = pz; ga.diag = diag;
        ga.xc[0] = xc[0]; ga.xc[1] = xc[1]; ga.xc[2] = xc[2];
        // the mixed mass-lumped step updates positions in the gather (no solve between them)
        ga.fuse_euler = std::is_same<R, float>::value && p.solver == FFEA_GPU_MASSLUMPED;
        ga.upx = px; ga.upy = py; ga.upz = pz; ga.uvx = vx; ga.uvy = vy; ga.uvz = vz; ga.dt = p.dt;
        if (ga.fuse_euler && fused_prep()) {
            ga.nu = me.u;
            ga.nvf = me.vf;
            ga.nxr = me.xr;
            // the gather closes the step: the next stream state into the other buffer
            ga.nrng = rng_state();
            ga.fin_jump = step_jump;
            ga.fin_next = rng_bufs[rng_cur ^ 1];
        }
        {
            NodeForces &sn = ga.sn;
            sn.noise = sn_chunk_jump != nullptr;
            sn.kT = p.kT;
            sn.dt = p.dt;
            sn.rng_state = rng_state();
            sn.chunk_jump = sn_chunk_jump;
            sn.lane_jump = sn_lane_jump;
            sn.node_orig = sn_node_orig;
            sn.node_drag = drag;
            sn.mid_orig = sn_mid_orig;
            sn.mid_drag = sn_mid_drag;
            ctf.fill(sn);
            sn.lin_ptr = sn_lin_ptr;
            sn.lin_ev = sn_lin_ev;
            sn.on = sn.noise || sn.lin_ptr != nullptr;
        }
        CK(ctf.launch(stream));
        // midpoints that carry force: each computed once (the vertices' linearise replay reads it up to ~20 times)
        const int M = (int)h.mid_nodes.size();
        if (ga.sn.lin_ptr && mid_f && (ga.sn.noise || ctf.mid || ctf.mface_ptr)) {
            CK(Launch<R>::mid_force(ga.sn, M, mid_f, st, stream));
            ga.sn.mid_f = mid_f;
        }
        int gblocks = gather_blocks;
        if (ga.nu && next_chunk_jump) {
            ga.ncj = next_chunk_jump;
            ga.nrng = rng_state();
            ga.nchunk_state = me.chunk_state;
            ga.nnchunks = me.nchunks;
            gblocks = std::max(gblocks, (me.nchunks + Launch<R>::gather_threads() - 1) / Launch<R>::gather_threads());
        }
        CK(Launch<R>::gather(ga, gblocks, stream));
        if ((rc = mark(3))) return rc;
        if (p.solver != FFEA_GPU_MASSLUMPED && (rc = launch_cg(init_partials, gather_blocks))) return rc;
        if ((rc = mark(4))) return rc;
        if (!ga.fuse_euler) {
            EulerArgs<R> eu{};
            eu.N = h.N; eu.nomass = nomass; eu.dt = p.dt; eu.x = x;
            eu.px = px; eu.py = py; eu.pz = pz; eu.vx = vx; eu.vy = vy; eu.vz = vz;
            eu.st = st;
            CK(Launch<R>::euler(eu, stream));
        }
        if (!ga.fin_next) CK(launch_finish_step(rng_state(), step_jump, st, stream));
        return mark(5);
    }

    int read_status(DevStatus &s) {
        CK(cudaMemcpyAsync(&s, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }

    int status_code(const DevStatus &s) {
        if (s.timeout) return FFEA_GPU_ETIMEOUT;
        if (s.inversions) return FFEA_GPU_EINVERTED;
        if (s.cg_fail) return FFEA_GPU_ECGMAXIT;
        if (s.nonfinite) return FFEA_GPU_ENAN;
        return FFEA_GPU_OK;
    }

    int step(int nsteps, int *done) override {
        if (nsteps < 0) return FFEA_GPU_EINPUT;
        DevStatus s{};
        int rc = read_status(s);
        if (rc) return rc;
        // clear the per-call flags, keep the CG totals
        s.inversions = s.cg_fail = s.nonfinite = s.timeout = s.abort = 0;
        s.steps_done = 0;
        CK(cudaMemcpyAsync(st, &s, sizeof(DevStatus), cudaMemcpyHostToDevice, stream));
        const int cur0 = rng_cur;
        for (int i = 0; i < nsteps; ++i) {
            rc = launch_step_graph(0, i > 0);
            if (rc) {
                settle_rng(cur0);
                return rc;
            }
            if (rng_bufs[1]) rng_cur ^= 1;
        }
        rc = read_status(s);
        if (rc) return rc;
        settle_rng(cur0, s.steps_done);
        if (done) *done = s.steps_done;
        return status_code(s);
    }

    // after a call's steps: with two stream buffers the current one follows the completed steps (a step that did
    // not complete wrote no next state); -1: read the count from the device
    void settle_rng(int cur0, int steps_done = -1) {
        if (!rng_bufs[1]) return;
        if (steps_done < 0) {
            DevStatus s{};
            if (read_status(s)) {
                rng_cur = cur0;
                return;
            }
            steps_done = s.steps_done;
        }
        rng_cur = (cur0 + steps_done) & 1;
    }

    int step_timed(int nsteps, long long flush_bytes, int *done, double *step_ms, double *phase_ms) override {
        if (nsteps < 0 || flush_bytes < 0) return FFEA_GPU_EINPUT;
        DevStatus s{};
        int rc = read_status(s);
        if (rc) return rc;
        s.inversions = s.cg_fail = s.nonfinite = s.timeout = s.abort = 0;
        s.steps_done = 0;
        CK(cudaMemcpyAsync(st, &s, sizeof(DevStatus), cudaMemcpyHostToDevice, stream));
        void *scratch = nullptr;
        if (flush_bytes > 0) CK(cudaMalloc(&scratch, (size_t)flush_bytes));
        double tot = 0.0, ph[FFEA_GPU_NUM_PHASES] = {0};
        const int cur0 = rng_cur;
        for (int i = 0; i < nsteps && rc == FFEA_GPU_OK; ++i) {
            if (scratch) {
                cudaError_t e = cudaMemsetAsync(scratch, i & 0xff, (size_t)flush_bytes, stream);
                if (e != cudaSuccess) { rc = cuda_fail(e, "flush"); break; }
            }
            if (phase_ms) {
                rc = launch_step_graph(1, i > 0);
            } else {  // the untimed graph, events around its launch only
                cudaError_t e = cudaEventRecord(ev[0], stream);
                if (e != cudaSuccess) { rc = cuda_fail(e, "cudaEventRecord"); break; }
                rc = launch_step_graph(0, i > 0);
                if (!rc && (e = cudaEventRecord(ev[FFEA_GPU_NUM_PHASES], stream)) != cudaSuccess)
                    rc = cuda_fail(e, "cudaEventRecord");
            }
            if (rc) break;
            if (rng_bufs[1]) rng_cur ^= 1;
            cudaError_t e = cudaEventSynchronize(ev[FFEA_GPU_NUM_PHASES]);
            if (e != cudaSuccess) { rc = cuda_fail(e, "cudaEventSynchronize"); break; }
            float ms = 0.f;
            if (phase_ms)
                for (int k = 0; k < FFEA_GPU_NUM_PHASES; ++k) {
                    cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
                    ph[k] += ms;
                }
            cudaEventElapsedTime(&ms, ev[0], ev[FFEA_GPU_NUM_PHASES]);
            tot += ms;
        }
        if (scratch) cudaFree(scratch);
        if (rc) {
            settle_rng(cur0);
            return rc;
        }
        rc = read_status(s);
        if (rc) return rc;
        settle_rng(cur0, s.steps_done);
        if (done) *done = s.steps_done;
        if (step_ms) *step_ms = tot;
        if (phase_ms)
            for (int k = 0; k < FFEA_GPU_NUM_PHASES; ++k) phase_ms[k] = ph[k];
        return status_code(s);
    }

    int get_state(double *pos, double *vel, double *force) override {
        const int N = h.N, n = h.n_all;
        // the reference layout is assembled on the device (midpoints as linearise_element leaves them) and
        // copied out in one transfer
        auto fill = [&](double *out, const double *dx, const double *dy, const double *dz, bool mids) -> int {
            CK(launch_aos_gather(dx, dy, dz, ref_src, n, mids ? 1 : 0, aos, stream));
            CK(cudaMemcpyAsync(out, aos, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            return FFEA_GPU_OK;
        };
        int rc;
        if (pos && (rc = fill(pos, px, py, pz, true))) return rc;
        if (vel && (rc = fill(vel, vx, vy, vz, false))) return rc;
        if (force) {
            std::vector<R> hxv(4 * (size_t)N);
            CK(cudaMemcpyAsync(hxv.data(), x, hxv.size() * sizeof(R), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            for (int i = 0; i < 3 * n; ++i) force[i] = 0.0;
            for (int k = 0; k < N; ++k)
                for (int c = 0; c < 3; ++c) force[3 * (size_t)h.node_of[k] + c] = (double)hxv[4 * (size_t)k + c];
        }
        return FFEA_GPU_OK;
    }

    int set_state(const double *pos, const double *vel) override {
        const int N = h.N;
        // one transfer of the reference-layout array, the vertex rows picked out on the device
        auto put = [&](const double *in, double *dx, double *dy, double *dz) -> int {
            CK(cudaMemcpyAsync(aos, in, 3 * (size_t)h.n_all * sizeof(double), cudaMemcpyHostToDevice, stream));
            CK(launch_aos_scatter(aos, d_node_of, N, dx, dy, dz, stream));
            return FFEA_GPU_OK;
        };
        int rc;
        if (vel && (rc = put(vel, vx, vy, vz))) return rc;
        if (pos && (rc = put(pos, px, py, pz))) return rc;
        if (pos) {
            // while the positions travel: the rigid modes must vanish at the pinned nodes' current positions, about
            // the new centroid (one pass over the vertex rows; the host copy of the positions is kept for the
            // pinned rows only)
            double s[3] = {0.0, 0.0, 0.0};
            for (int k = 0; k < N; ++k) {
                const double *q = pos + 3 * (size_t)h.node_of[k];
                s[0] += q[0]; s[1] += q[1]; s[2] += q[2];
                if (h.pinned[k])
                    for (int c = 0; c < 3; ++c) h.pos[3 * (size_t)k + c] = q[c];
            }
            for (int c = 0; c < 3; ++c) xc[c] = s[c] / std::max(N, 1);
            nmodes = rigid_modes_about(h, p, xc, modes, 0, N);
            // the gather and the CG take the centroid and the modes by value
            for (auto &r : refresh) r = true;
        }
        // the caller may reuse its arrays on return
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }

    int set_rng(const uint32_t s[6]) override {
        CK(cudaMemcpyAsync(rng_state(), s, 6 * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }

    int get_rng(uint32_t s[6]) override {
        CK(cudaMemcpyAsync(s, rng_state(), 6 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }

    int cg_iters(int *last, long long *total) override {
        DevStatus s{};
        int rc = read_status(s);
        if (rc) return rc;
        if (last) *last = s.last_iters;
        if (total) *total = s.total_iters;
        return FFEA_GPU_OK;
    }

    int get_elements(double *nf, double *vol, double *visc) override {
        if constexpr (std::is_same<R, float>::value) {
            g_last_error = "per-element outputs are kept by the FP64 path only (the mixed path sums each thread "
                           "block's element forces per vertex)";
            return FFEA_GPU_EINPUT;
        }
        const int T = h.T;
        std::vector<R> he(12 * (size_t)T), hg(16 * (size_t)T);
        CK(cudaMemcpyAsync(he.data(), ef, he.size() * sizeof(R), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(hg.data(), geom, hg.size() * sizeof(R), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (nf)
            for (size_t i = 0; i < he.size(); ++i) nf[i] = (double)he[i];
        if (vol)
            for (int e = 0; e < T; ++e) vol[e] = (double)hg[16 * (size_t)e + 12];
        if (visc)
            for (int e = 0; e < T; ++e) {
                double d[12];
                for (int k = 0; k < 12; ++k) d[k] = (double)hg[16 * (size_t)e + k];
                const double v = (double)hg[16 * (size_t)e + 12];
                for (int rr = 0; rr < 12; ++rr)
                    for (int cc = 0; cc < 12; ++cc)
                        visc[144 * (size_t)e + 12 * rr + cc] =
                            host_visc_entry(d, (double)(R)h.A[e], (double)(R)h.B[e], v, rr, cc);
            }
        return FFEA_GPU_OK;
    }

    int cg_history(double *res2, int max_entries, int *count) override {
        DevStatus s{};
        int rc = read_status(s);
        if (rc) return rc;
        const int n = std::max(0, std::min({s.last_iters, hist_cap, max_entries}));
        if (n > 0 && res2) {
            CK(cudaMemcpyAsync(res2, history, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
        }
        if (count) *count = n;
        return FFEA_GPU_OK;
    }

    int cg_profile(double *ns, int n) override {
        unsigned long long t[FFEA_GPU_CG_PHASES];
        CK(cudaMemcpyAsync(t, phase_ns, sizeof t, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        for (int k = 0; k < n && k < FFEA_GPU_CG_PHASES; ++k) ns[k] = (double)t[k];
        return FFEA_GPU_OK;
    }

    int cg_preconditioner(int *degree, double *lambda_max) override {
        double c = 0.0;
        if (cheb) {
            CK(cudaMemcpyAsync(&c, cheb, sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
        }
        if (degree) *degree = c > 0.0 ? cg_poly : 0;
        if (lambda_max) *lambda_max = c > 0.0 ? c : 0.0;
        return FFEA_GPU_OK;
    }

    const char *cg_kernel_name() const override {
        if (p.solver == FFEA_GPU_MASSLUMPED) return "none";
        if constexpr (std::is_same<R, float>::value) {
            if (cg_npb > 0 && cg_sr && p.solver == FFEA_GPU_NOMASS_CG) return "cg_mixed_sr_kernel";
            return cg_npb > 0 ? "cg_mixed_own_kernel" : "cg_mixed_kernel";
        } else {
            return cg_npb > 0 ? "cg_own_kernel" : "cg_kernel";
        }
    }

    int get_rhs(double *rhs) override {
        const int N = h.N;
        std::vector<double> hf(4 * (size_t)N);
        if (f32) {
            std::vector<float> h32(4 * (size_t)N);
            CK(cudaMemcpyAsync(h32.data(), f32, h32.size() * sizeof(float), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            for (size_t i = 0; i < h32.size(); ++i) hf[i] = h32[i];
        } else {
            CK(cudaMemcpyAsync(hf.data(), f, hf.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
        }
        for (int i = 0; i < 3 * h.n_all; ++i) rhs[i] = 0.0;
        for (int k = 0; k < N; ++k)
            for (int c = 0; c < 3; ++c) rhs[3 * (size_t)h.node_of[k] + c] = hf[4 * (size_t)k + c];
        return FFEA_GPU_OK;
    }

    int get_matrix_values(std::vector<double> &out) override {
        const bool block3 = p.solver == FFEA_GPU_NOMASS_CG;
        std::vector<R> hv((block3 ? 9 : 1) * (size_t)h.nslots);
        CK(cudaMemcpyAsync(hv.data(), val, hv.size() * sizeof(R), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        out.assign(hv.begin(), hv.end());
        return FFEA_GPU_OK;
    }

    // Jacobi-PCG solve of the blob's current matrix with every work array in g_solve_scratch, by the
    // grid-strided cg_kernel opened by solve_static_prep_kernel instead of the gather. A step of a blob whose
    // rows fit in shared memory runs cg_own_kernel instead, whose sums run in another order, so the two agree
    // to rounding, not bit for bit. Host copies go through the blob's pinned staging buffer; nothing is
    // allocated. The blob's device is current for the call (the caller's is restored), and once a kernel is
    // queued every return waits for the stream first, so the lock is never released while a kernel of this
    // call may still use the shared array.
    int solve_static(const double *rhs, double *xout, int *iterations) override {
        if constexpr (std::is_same<R, float>::value) {
            g_last_error = "ffea_gpu_blob_solve_static: FP64 blobs only";
            return FFEA_GPU_EINPUT;
        } else {
            if (p.solver == FFEA_GPU_MASSLUMPED) {
                g_last_error = "ffea_gpu_blob_solve_static: the mass-lumped solver has no CG solve";
                return FFEA_GPU_EINPUT;
            }
            const int N = h.N;
            if (N > SOLVE_STATIC_MAX_NODES || cg_grid > SOLVE_MAX_BLOCKS) {
                g_last_error = "ffea_gpu_blob_solve_static: " + std::to_string(N) +
                               " vertex nodes exceed the static scratch limit of " +
                               std::to_string(SOLVE_STATIC_MAX_NODES);
                return FFEA_GPU_EINPUT;
            }
            std::lock_guard<std::mutex> lock(g_solve_mutex);
            int caller_device = -1;
            CK(cudaGetDevice(&caller_device));
            struct RestoreDevice {
                int d;
                ~RestoreDevice() { cudaSetDevice(d); }
            } restore_device{caller_device};
            if (caller_device != device) CK(cudaSetDevice(device));
            double *s = nullptr;
            int rc = solve_scratch(device, &s);
            if (rc) return rc;
            CK(cudaStreamSynchronize(stream));  // staging may still feed an earlier copy
            // declared after the lock, so destroyed before it: no early return leaves a kernel running
            struct SyncOnExit {
                cudaStream_t st;
                ~SyncOnExit() { cudaStreamSynchronize(st); }
            } sync_on_exit{stream};
            for (int k = 0; k < N; ++k)
                for (int c = 0; c < 3; ++c) staging[3 * (size_t)k + c] = rhs[3 * (size_t)h.node_of[k] + c];
            CK(cudaMemcpyAsync(s + SS_RHS, staging, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, stream));
            const int blocks = (N + SOLVE_PREP_THREADS - 1) / SOLVE_PREP_THREADS;
            GridBarrier *sgb = reinterpret_cast<GridBarrier *>(s + SS_BARRIER);
            DevStatus *sst = reinterpret_cast<DevStatus *>(s + SS_STATUS);
            unsigned long long *sphase = reinterpret_cast<unsigned long long *>(s + SS_PHASE);
            solve_static_prep_kernel<<<blocks, SOLVE_PREP_THREADS, 0, stream>>>(
                N, s + SS_RHS, dinv, s + SS_X, s + SS_R, s + SS_INIT, SOLVE_MAX_BLOCKS, sgb, sst, sphase);
            count_launch();
            CK(cudaGetLastError());
            const bool nomass = p.solver == FFEA_GPU_NOMASS_CG;
            CgArgs<R> ca{};
            ca.N = N;
            ca.block3 = nomass;
            ca.check_last = nomass;
            ca.slice_ptr = slice_ptr; ca.rowlen = rowlen; ca.bcol = bcol;
            ca.val = val; ca.dinv = dinv;
            ca.x = s + SS_X; ca.r = s + SS_R; ca.q = s + SS_Q; ca.pbuf0 = s + SS_P; ca.pbuf1 = nullptr;
            ca.init_partials = s + SS_INIT; ca.n_init = blocks; ca.init_stride = SOLVE_MAX_BLOCKS;
            ca.partials = s + SS_PART; ca.stride = SOLVE_MAX_BLOCKS;
            ca.gb = sgb; ca.st = sst;
            ca.imax = p.max_iterations_cg;
            ca.eps2 = p.epsilon2;
            ca.limit_ns = 2000000000ull;
            ca.history = nullptr; ca.hist_cap = 0; ca.tpn = tpn; ca.phase_ns = sphase;
            CK(Launch<R>::cg(ca, cg_grid, cg_block, stream));
            DevStatus ds{};
            CK(cudaMemcpy2DAsync(staging, 3 * sizeof(double), s + SS_X, 4 * sizeof(double), 3 * sizeof(double), N,
                                 cudaMemcpyDeviceToHost, stream));
            CK(cudaMemcpyAsync(&ds, sst, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            if (iterations) *iterations = ds.last_iters;
            if ((rc = status_code(ds))) return rc;
            // midpoint rows are identity rows of the reference's system; rhs and xout may be one array
            for (int i = 0; i < h.n_all; ++i)
                if (h.lin_of[i] < 0)
                    for (int c = 0; c < 3; ++c) xout[3 * (size_t)i + c] = rhs[3 * (size_t)i + c];
            for (int k = 0; k < N; ++k)
                for (int c = 0; c < 3; ++c) xout[3 * (size_t)h.node_of[k] + c] = staging[3 * (size_t)k + c];
            return FFEA_GPU_OK;
        }
    }

    int upload_linearise(Arena &m) {
        CK(m.upload(&sn_lin_ptr, h.lin_ptr));
        std::vector<int4> ev(h.lin_ev.size() / 4);
        for (size_t k = 0; k < ev.size(); ++k)
            ev[k] = make_int4(h.lin_ev[4 * k], h.lin_ev[4 * k + 1], h.lin_ev[4 * k + 2], -1);
        CK(m.upload(&sn_lin_ev, ev));
        return FFEA_GPU_OK;
    }

    int load_ctforces(const char *ctf_file, const char *surf_file, int blob_index) override {
        invalidate_graphs();
        CtfModel cm;
        std::string err;
        int rc = ffea::host::load_ctforces(ctf_file, surf_file, blob_index, h.n_all, cm, err);
        if (rc) {
            g_last_error = err;
            return rc;
        }
        if (lin_from_ctf) {  // the replay lived with the previous constant forces
            sn_lin_ptr = nullptr;
            sn_lin_ev = nullptr;
            lin_mem.clear();
            lin_from_ctf = false;
        }
        CK(ctf.build(h, cm, px, py, pz, st));
        const int M = (int)h.mid_nodes.size();
        if (ctf.mid_force && !mid_f && M > 0) CK(mem.alloc(&mid_f, 3 * (size_t)M));
        // midpoints that carry force need the linearisation replay (already there with Stokes noise)
        if (ctf.mid_force && !sn_lin_ptr) {
            build_linearise_events(h);
            int lrc = upload_linearise(lin_mem);
            if (lrc) return lrc;
            lin_from_ctf = true;
        }
        return FFEA_GPU_OK;
    }

    // the step's stream advance, and where the Stokes draws start (node i of the reference numbering draws
    // 3 numbers from stokes_base + 3i after the step's state)
    int set_rng_layout(unsigned long long step_draws, unsigned long long stokes_base) override {
        invalidate_graphs();
        std::vector<MrgJump> sj(1, jump_pow(step_draws));
        CK(cudaMemcpy(step_jump, sj.data(), sizeof(MrgJump), cudaMemcpyHostToDevice));
        int nrc = upload_next_chunk_jumps(step_draws);
        if (nrc) return nrc;
        if (sn_chunk_jump) {
            const int nch = (h.n_all + 31) / 32;
            std::vector<MrgJump> ncj(nch);
            const Mat3 a96 = mat_pow(MRG_A1, 96, MRG_M1), b96 = mat_pow(MRG_A2, 96, MRG_M2);
            Mat3 ca = mat_pow(MRG_A1, stokes_base, MRG_M1), cb = mat_pow(MRG_A2, stokes_base, MRG_M2);
            for (int c = 0; c < nch; ++c) {
                ncj[c] = to_jump(ca, cb);
                ca = mat_mul(a96, ca, MRG_M1);
                cb = mat_mul(b96, cb, MRG_M2);
            }
            CK(cudaMemcpy(sn_chunk_jump, ncj.data(), ncj.size() * sizeof(MrgJump), cudaMemcpyHostToDevice));
        }
        return FFEA_GPU_OK;
    }

    // ---- adjoint window ---------------------------------------------------------------------
    int adj_init(int window, int every) override {
        if (p.solver != FFEA_GPU_NOMASS_CG) {
            g_last_error = "the adjoint covers the CG_nomass solver";
            return FFEA_GPU_EINPUT;
        }
        if (window <= 0 || every <= 0) {
            g_last_error = "adjoint window and checkpoint interval must be positive";
            return FFEA_GPU_EINPUT;
        }
        if (ctf.any) {
            g_last_error = "the adjoint does not differentiate constant forces";
            return FFEA_GPU_EINPUT;
        }
        adj_release();
        adj_mem.reset(new Arena());
        const int N = h.N, T = h.T, nck = (window + every - 1) / every, seg = std::min(every, window);
        Arena &m = *adj_mem;
        CK(m.alloc(&ck_pos, 3 * (size_t)N * nck));
        CK(m.alloc(&ck_det, (size_t)T * nck));
        CK(m.alloc(&ck_rng, 6 * (size_t)nck));
        CK(m.alloc(&seg_pos, 3 * (size_t)N * seg));
        CK(m.alloc(&seg_v, 4 * (size_t)N * seg));
        CK(m.alloc(&seg_rng, 6 * (size_t)seg));
        CK(m.alloc(&lam, 4 * (size_t)N));
        CK(m.alloc(&eg, 12 * (size_t)T));
        CK(m.alloc(&gtheta, 4 * (size_t)T));
        CK(m.alloc(&coef, 6));
        CK(m.alloc(&adj_part_d, (size_t)ADJ_MOMENTS * gather_blocks));
        CK(m.alloc(&adj_part_f, (size_t)ADJ_MOMENTS * gather_blocks));
        CK(m.alloc(&fin_pos, 3 * (size_t)N));
        CK(m.alloc(&fin_det, (size_t)T));
        CK(m.alloc(&fin_rng, 6));
        adj_window = window;
        adj_every = every;
        adj_done = -1;
        return FFEA_GPU_OK;
    }

    void adj_release() override {
        adj_mem.reset();
        adj_window = adj_every = 0;
        adj_done = -1;
    }

    // device copies of the state a step depends on: positions (SoA), stream state, last determinants
    int save_state(double *pos3, uint32_t *rng, double *det) {
        const size_t N = h.N;
        CK(cudaMemcpyAsync(pos3, px, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(pos3 + N, py, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(pos3 + 2 * N, pz, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        if (rng) CK(cudaMemcpyAsync(rng, rng_state(), 6 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
        if (det) CK(cudaMemcpyAsync(det, last_det, h.T * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        return FFEA_GPU_OK;
    }

    int load_state(const double *pos3, const uint32_t *rng, const double *det) {
        const size_t N = h.N;
        CK(cudaMemcpyAsync(px, pos3, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(py, pos3 + N, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(pz, pos3 + 2 * N, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        if (rng) CK(cudaMemcpyAsync(rng_state(), rng, 6 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
        if (det) CK(cudaMemcpyAsync(last_det, det, h.T * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        return FFEA_GPU_OK;
    }

    int clear_flags() {
        DevStatus s{};
        int rc = read_status(s);
        if (rc) return rc;
        s.inversions = s.cg_fail = s.nonfinite = s.timeout = s.abort = 0;
        s.steps_done = 0;
        CK(cudaMemcpyAsync(st, &s, sizeof(DevStatus), cudaMemcpyHostToDevice, stream));
        return FFEA_GPU_OK;
    }

    // the window's forward pass: `adj_window` steps from the current state, a checkpoint every
    // `adj_every` steps (positions, stream state, last determinants before the step)
    int adj_forward(int *done) override {
        if (!adj_mem) return FFEA_GPU_EINPUT;
        int rc = clear_flags();
        if (rc) return rc;
        const size_t N = h.N;
        for (int n = 0; n < adj_window; ++n) {
            if (n % adj_every == 0) {
                const int c = n / adj_every;
                if ((rc = save_state(ck_pos + 3 * N * c, ck_rng + 6 * c, ck_det + (size_t)h.T * c))) return rc;
            }
            if ((rc = launch_step())) return rc;
        }
        DevStatus s{};
        if ((rc = read_status(s))) return rc;
        if (done) *done = s.steps_done;
        adj_done = s.steps_done;
        return status_code(s);
    }

    // one backward step at stored positions and stream state: lambda <- lambda + d(dt v)/dx^T lambda,
    // gtheta += d(dt v)/dtheta^T lambda
    int adj_step(const R *v_step) {
        constexpr bool mixed = std::is_same<R, float>::value;
        int rc = launch_elements(1);
        if (rc) return rc;
        rc = launch_assemble();
        if (rc) return rc;
        AdjGatherArgs<R> ag{};
        ag.N = h.N;
        ag.dt = p.dt;
        ag.lam = lam;
        ag.pinned = pinned;
        ag.px = px; ag.py = py; ag.pz = pz;
        for (int c = 0; c < 3; ++c) ag.xc[c] = xc[c];
        ag.dinv = dinv;
        ag.diag = mixed ? diag : nullptr;
        ag.f = f; ag.r = r; ag.x = x;
        ag.dpos = mixed ? dpos : nullptr;
        ag.partials_d = mixed ? nullptr : adj_part_d;
        ag.partials_f = mixed ? adj_part_f : nullptr;
        ag.stride = gather_blocks;
        ag.gb = gb;
        ag.st = st;
        CK(AdjLaunch<R>::gather(ag, gather_blocks, stream));
        AdjModesArgs am{};
        am.partials_d = mixed ? nullptr : adj_part_d;
        am.partials_f = mixed ? adj_part_f : nullptr;
        am.stride = gather_blocks;
        am.nb = gather_blocks;
        am.nmodes = nmodes;
        for (int i = 0; i < 36; ++i) am.modes[i] = modes[i];
        am.coef = coef;
        CK(AdjLaunch<R>::modes(am, stream));
        if (mixed) {
            // cg_mixed_kernel projects the right-hand side itself from the moments
            if ((rc = launch_cg(reinterpret_cast<const double *>(adj_part_f), gather_blocks))) return rc;
        } else {
            AdjApplyArgs<R> aa{};
            aa.N = h.N;
            aa.px = px; aa.py = py; aa.pz = pz;
            for (int c = 0; c < 3; ++c) aa.xc[c] = xc[c];
            aa.coef = coef;
            aa.dinv = dinv;
            aa.r = r;
            aa.f = f;
            aa.partials = init_partials;
            aa.stride = gather_blocks;
            aa.st = st;
            CK(AdjLaunch<R>::apply(aa, gather_blocks, stream));
            if ((rc = launch_cg(init_partials, gather_blocks))) return rc;
        }
        AdjElemArgs<R> ae{};
        ae.T = h.T;
        ae.calc_noise = p.calc_noise;
        ae.kT = p.kT;
        ae.dt = p.dt;
        ae.tet = tet;
        ae.px = px; ae.py = py; ae.pz = pz;
        ae.jinv = jinv; ae.G = G; ae.E = E; ae.A = A; ae.B = B; ae.vol0 = vol0;
        ae.rng_state = rng_state(); ae.chunk_jump = chunk_jump; ae.lane_jump = lane_jump;
        ae.mu = x;
        ae.v = v_step;
        ae.nmodes = nmodes;
        for (int c = 0; c < 3; ++c) ae.xc[c] = xc[c];
        ae.coef = coef;
        ae.eg = eg;
        ae.gtheta = gtheta;
        ae.st = st;
        CK(AdjLaunch<R>::elem(ae, stream));
        AdjNodeArgs<R> an{};
        an.N = h.N;
        an.inc_ptr = inc_ptr; an.inc = inc;
        an.eg = eg;
        an.v = v_step;
        an.dinv = dinv;
        an.diag = mixed ? diag : nullptr;
        an.nmodes = nmodes;
        an.coef = coef;
        an.lam = lam;
        an.st = st;
        CK(AdjLaunch<R>::node(an, stream));
        return FFEA_GPU_OK;
    }

    int adj_backward(const double *dl_dx, double *dG, double *dE, double *dA, double *dB,
                     double *dl_dx0) override {
        if (!adj_mem || adj_done != adj_window) {
            g_last_error = "run the adjoint window's forward pass first";
            return FFEA_GPU_EINPUT;
        }
        const int N = h.N, T = h.T;
        // dL/dx_final on vertex rows: a midpoint's share goes half to each edge end
        std::vector<double> l4(4 * (size_t)N, 0.0);
        for (int k = 0; k < N; ++k)
            for (int c = 0; c < 3; ++c) l4[4 * (size_t)k + c] = dl_dx[3 * (size_t)h.node_of[k] + c];
        for (size_t m = 0; m < h.mid_nodes.size(); ++m)
            for (int c = 0; c < 3; ++c) {
                const double gm = 0.5 * dl_dx[3 * (size_t)h.mid_nodes[m] + c];
                l4[4 * (size_t)h.mid_a[m] + c] += gm;
                l4[4 * (size_t)h.mid_b[m] + c] += gm;
            }
        CK(cudaMemcpyAsync(lam, l4.data(), l4.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        CK(cudaMemsetAsync(gtheta, 0, 4 * (size_t)T * sizeof(double), stream));
        DevStatus s0{};
        int rc = read_status(s0);
        if (rc) return rc;
        if ((rc = save_state(fin_pos, fin_rng, fin_det))) return rc;
        if ((rc = clear_flags())) return rc;
        const size_t N3 = 3 * (size_t)N, N4 = 4 * (size_t)N;
        const int nseg = (adj_window + adj_every - 1) / adj_every;
        for (int sg = nseg - 1; sg >= 0 && !rc; --sg) {
            const int c0 = sg * adj_every, len = std::min(adj_every, adj_window - c0);
            if ((rc = load_state(ck_pos + N3 * sg, ck_rng + 6 * sg, ck_det + (size_t)T * sg))) break;
            for (int j = 0; j < len && !rc; ++j) {  // recompute the segment, keeping x_n, v_n, stream states
                if ((rc = save_state(seg_pos + N3 * j, seg_rng + 6 * j, nullptr))) break;
                if ((rc = launch_step())) break;
                cudaError_t e = cudaMemcpyAsync(seg_v + N4 * j, x, N4 * sizeof(R), cudaMemcpyDeviceToDevice, stream);
                if (e != cudaSuccess) rc = cuda_fail(e, "segment velocity copy");
            }
            for (int j = len - 1; j >= 0 && !rc; --j) {
                if ((rc = load_state(seg_pos + N3 * j, seg_rng + 6 * j, nullptr))) break;
                rc = adj_step(seg_v + N4 * j);
            }
        }
        DevStatus s{};
        if (!rc) rc = read_status(s);
        if (!rc) rc = status_code(s);
        if (!rc) {
            std::vector<double> gt(4 * (size_t)T);
            CK(cudaMemcpyAsync(gt.data(), gtheta, gt.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaMemcpyAsync(l4.data(), lam, l4.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            for (int e = 0; e < T; ++e) {
                if (dG) dG[e] = gt[4 * (size_t)e];
                if (dE) dE[e] = gt[4 * (size_t)e + 1];
                if (dA) dA[e] = gt[4 * (size_t)e + 2];
                if (dB) dB[e] = gt[4 * (size_t)e + 3];
            }
            if (dl_dx0) {
                for (int i = 0; i < 3 * h.n_all; ++i) dl_dx0[i] = 0.0;
                for (int k = 0; k < N; ++k)
                    for (int c = 0; c < 3; ++c) dl_dx0[3 * (size_t)h.node_of[k] + c] = l4[4 * (size_t)k + c];
            }
        }
        // the blob continues from the end of the window
        int rc2 = load_state(fin_pos, fin_rng, fin_det);
        if (!rc2) {
            CK(cudaMemcpyAsync(st, &s0, sizeof(DevStatus), cudaMemcpyHostToDevice, stream));
            CK(cudaStreamSynchronize(stream));
        }
        return rc ? rc : rc2;
    }

    // Blob::make_measurements energies (src/Blob.cpp:1066-1125), evaluated on the host from device state
    // Blob::make_measurements on the device: out = strain energy, kinetic energy, centroid (3) of all nodes,
    // RMSD of all nodes from the reference positions (meso units)
    int measurements(double out[MEASURE_NV]) override {
        MeasureArgs<R> ma{};
        ma.T = h.T;
        ma.N = h.N;
        ma.M = (int)h.mid_nodes.size();
        ma.inertial = p.solver != FFEA_GPU_NOMASS_CG;
        ma.tet = tet;
        ma.px = px; ma.py = py; ma.pz = pz; ma.vx = vx; ma.vy = vy; ma.vz = vz;
        ma.jinv = jinv; ma.G = G; ma.E = E; ma.vol0 = vol0; ma.rho = rho;
        ma.p0 = p0; ma.mid_a = mid_a; ma.mid_b = mid_b; ma.m0 = m0;
        ma.partials = meas_part;
        CK(Launch<R>::measure(ma, meas_blocks, meas_out, stream));
        double s6[MEASURE_NV];
        CK(cudaMemcpyAsync(s6, meas_out, sizeof s6, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        const double n = (double)std::max(h.n_all, 1);
        out[0] = s6[0];
        out[1] = s6[1];
        out[2] = s6[2] / n;
        out[3] = s6[3] / n;
        out[4] = s6[4] / n;
        out[5] = sqrt(s6[5] / n);
        return FFEA_GPU_OK;
    }

    int measure(double *se, double *ke) override {
        double o[MEASURE_NV];
        int rc = measurements(o);
        if (rc) return rc;
        if (se) *se = o[0];
        if (ke) *ke = o[1];
        return FFEA_GPU_OK;
    }

    // Blob::set_pos_0: the current positions become the RMSD reference
    int set_rmsd_reference() override {
        const int N = h.N, M = (int)h.mid_nodes.size();
        std::vector<double> q(3 * (size_t)N), qm(3 * (size_t)std::max(M, 1));
        CK(cudaMemcpyAsync(q.data(), px, N * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(q.data() + N, py, N * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(q.data() + 2 * (size_t)N, pz, N * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        for (int m = 0; m < M; ++m)
            for (int c = 0; c < 3; ++c)
                qm[(size_t)c * M + m] = .5 * (q[(size_t)c * N + h.mid_a[m]] + q[(size_t)c * N + h.mid_b[m]]);
        CK(cudaMemcpyAsync(p0, q.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(m0, qm.data(), qm.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }
};

static_assert(FFEA_GPU_CG_POLY_MAX == CHEB_MAX, "the CG kernel holds the coefficients of every accepted degree");
static_assert(FFEA_GPU_CG_POLY_DEFAULT > 0 && FFEA_GPU_CG_POLY_DEFAULT <= CHEB_MAX && FFEA_GPU_CG_POLY_DEFAULT % 2 == 0,
              "the default Chebyshev degree is an accepted one");

int check_params(const ffea_gpu_params *p) {
    if (!p) return FFEA_GPU_EINPUT;
    if (p->solver < 0 || p->solver > 2 || (p->precision != FFEA_GPU_FP64 && p->precision != FFEA_GPU_MIXED) ||
        p->max_iterations_cg < 0 || !(p->dt > 0) ||
        (p->cg_poly < -1 || p->cg_poly > FFEA_GPU_CG_POLY_MAX || (p->cg_poly > 0 && p->cg_poly % 2 != 0)) || p->cg_smem_blocks < -1) {
        g_last_error = "invalid parameters";
        return FFEA_GPU_EINPUT;
    }
    return FFEA_GPU_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int ffea_gpu_params_default(ffea_gpu_params *p) {
    if (!p) return FFEA_GPU_EINPUT;
    std::memset(p, 0, sizeof(*p));
    p->dt = 1e-14 / MESO_TIME;
    p->kT = 4.11e-21 / MESO_ENERGY;
    p->epsilon2 = 0.01;
    p->stokes_visc = 1e-3 / (MESO_PRESSURE * MESO_TIME);
    p->max_iterations_cg = 1000;
    p->calc_noise = 1;
    p->calc_stokes = 1;
    p->solver = FFEA_GPU_NOMASS_CG;
    p->precision = FFEA_GPU_FP64;
    return FFEA_GPU_OK;
}

int ffea_gpu_material_from_si(int n, const double *mat6, double *rho, double *A, double *B, double *G, double *E) {
    if (n < 0 || (n > 0 && !mat6)) return FFEA_GPU_EINPUT;
    for (int e = 0; e < n; ++e) {
        const double *m = mat6 + 6 * (size_t)e;
        if (rho) rho[e] = m[0] * MESO_VOLUME / MESO_MASS;
        if (A) A[e] = m[1] / (MESO_PRESSURE * MESO_TIME);
        if (B) B[e] = m[2] / (MESO_PRESSURE * MESO_TIME) - (2.0 / 3.0) * m[1];
        if (G) G[e] = m[3] / MESO_PRESSURE;
        if (E) E[e] = m[4] / MESO_PRESSURE;
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_blob_create(const ffea_gpu_mesh *mesh, const ffea_gpu_params *params, ffea_gpu_blob **out) {
    if (!out || !mesh) return FFEA_GPU_EINPUT;
    *out = nullptr;
    int rc = check_params(params);
    if (rc) return rc;
    ffea_gpu_blob *b = nullptr;
    try {
        if (params->precision == FFEA_GPU_MIXED) b = new BlobImpl<float>();
        else b = new BlobImpl<double>();
    } catch (std::bad_alloc &) {
        return FFEA_GPU_ENOMEM;
    }
    b->p = *params;
    try {
        rc = build_model(mesh, params, b->h);
    } catch (std::bad_alloc &) {
        rc = FFEA_GPU_ENOMEM;
    }
    if (!rc) rc = b->init();
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return FFEA_GPU_OK;
}

void ffea_gpu_blob_destroy(ffea_gpu_blob *blob) { delete blob; }

int ffea_gpu_blob_set_rng_state(ffea_gpu_blob *b, const uint32_t s[6]) {
    if (!b || !s || !valid_seed(s)) return FFEA_GPU_EINPUT;
    return b->set_rng(s);
}

int ffea_gpu_blob_get_rng_state(ffea_gpu_blob *b, uint32_t s[6]) {
    if (!b || !s) return FFEA_GPU_EINPUT;
    return b->get_rng(s);
}

int ffea_gpu_blob_step(ffea_gpu_blob *b, int nsteps, int *done) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->step(nsteps, done);
}

int ffea_gpu_blob_step_timed(ffea_gpu_blob *b, int nsteps, long long flush_bytes, int *done, double *step_ms,
                             double *phase_ms) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->step_timed(nsteps, flush_bytes, done, step_ms, phase_ms);
}

int ffea_gpu_blob_get_state(ffea_gpu_blob *b, double *pos, double *vel, double *force) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->get_state(pos, vel, force);
}

int ffea_gpu_blob_set_state(ffea_gpu_blob *b, const double *pos, const double *vel) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->set_state(pos, vel);
}

int ffea_gpu_blob_measure(ffea_gpu_blob *b, double *se, double *ke) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->measure(se, ke);
}

int ffea_gpu_blob_load_ctforces(ffea_gpu_blob *b, const char *ctforces_file, const char *surface_file,
                                int blob_index) {
    if (!b || !ctforces_file || blob_index < 0) return FFEA_GPU_EINPUT;
    return b->load_ctforces(ctforces_file, surface_file, blob_index);
}

int ffea_gpu_blob_measurements(ffea_gpu_blob *b, double out[6]) {
    if (!b || !out) return FFEA_GPU_EINPUT;
    return b->measurements(out);
}

int ffea_gpu_blob_set_rmsd_reference(ffea_gpu_blob *b) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->set_rmsd_reference();
}

int ffea_gpu_blob_cg_iterations(ffea_gpu_blob *b, int *last, long long *total) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->cg_iters(last, total);
}

int ffea_gpu_blob_cg_history(ffea_gpu_blob *b, double *res2, int max_entries, int *count) {
    if (!b || max_entries < 0) return FFEA_GPU_EINPUT;
    return b->cg_history(res2, max_entries, count);
}

int ffea_gpu_blob_cg_profile(ffea_gpu_blob *b, double *ns, int n) {
    if (!b || !ns || n < 0) return FFEA_GPU_EINPUT;
    if (b->p.solver == FFEA_GPU_MASSLUMPED) {
        for (int k = 0; k < n; ++k) ns[k] = 0.0;
        return FFEA_GPU_OK;
    }
    return b->cg_profile(ns, n);
}

int ffea_gpu_blob_cg_preconditioner(ffea_gpu_blob *b, int *degree, double *lambda_max) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->cg_preconditioner(degree, lambda_max);
}

const char *ffea_gpu_blob_cg_kernel(ffea_gpu_blob *b) { return b ? b->cg_kernel_name() : "none"; }

int ffea_gpu_blob_counts(ffea_gpu_blob *b, int *num_nodes, int *num_elements) {
    if (!b) return FFEA_GPU_EINPUT;
    if (num_nodes) *num_nodes = b->h.n_all;
    if (num_elements) *num_elements = b->h.T;
    return FFEA_GPU_OK;
}

int ffea_gpu_blob_sizes(ffea_gpu_blob *b, int *nl, int *ne, long long *nb) {
    if (!b) return FFEA_GPU_EINPUT;
    if (nl) *nl = b->h.N;
    if (ne) *ne = b->h.T;
    if (nb) {
        long long s = 0;
        for (int a = 0; a < b->h.N; ++a) s += b->h.rowlen[a];
        *nb = s;
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_blob_get_pattern(ffea_gpu_blob *b, int *key, int *col, double *val, int *nsrc, long long *nnz) {
    if (!b) return FFEA_GPU_EINPUT;
    const HostModel &h = b->h;
    if (b->p.solver != FFEA_GPU_NOMASS_CG) return FFEA_GPU_EINPUT;
    const int n = h.n_all;
    // rows of the reference: vertex rows carry 3 entries per neighbour block, others one diagonal entry
    std::vector<int> len(n, 1);
    for (int k = 0; k < h.N; ++k)
        if (!h.pinned[k]) len[h.node_of[k]] = 3 * h.rowlen[k];
    long long total = 0;
    for (int i = 0; i < n; ++i) total += 3ll * len[i];
    if (nnz) *nnz = total;
    if (!col && !key && !val && !nsrc) return FFEA_GPU_OK;
    std::vector<double> vals;
    if (val) {
        int rc = b->get_matrix_values(vals);
        if (rc) return rc;
    }
    long long pos = 0;
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            if (key) key[3 * (size_t)i + c] = (int)pos;
            const int k = h.lin_of[i];
            if (k >= 0 && !h.pinned[k]) {
                const int s = k >> 5, lane = k & 31;
                for (int m = 0; m < h.rowlen[k]; ++m) {
                    const long long slot = (long long)h.slice_ptr[s] + 32 * m + lane;
                    const int bcolv = h.bcol[slot];
                    const int nsource = h.src_ptr[slot + 1] - h.src_ptr[slot];
                    for (int j = 0; j < 3; ++j) {
                        if (col) col[pos] = 3 * h.node_of[bcolv] + j;
                        if (val) val[pos] = vals[9 * (size_t)h.slice_ptr[s] + 32 * (9 * m + 3 * c + j) + lane];
                        if (nsrc) nsrc[pos] = nsource + ((m == h.diagk[k] && c == j && b->p.calc_stokes == 1) ? 1 : 0);
                        ++pos;
                    }
                }
            } else {
                // pinned vertex or midpoint: the identity `one` (+ Stokes drag on unpinned midpoints)
                const bool stokes = b->p.calc_stokes == 1 && !h.pinned_all[i];
                if (col) col[pos] = 3 * i + c;
                if (val) val[pos] = 1.0 + (stokes ? h.drag_all[i] : 0.0);
                if (nsrc) nsrc[pos] = 1 + (stokes ? 1 : 0);
                ++pos;
            }
        }
    if (key) key[3 * (size_t)n] = (int)pos;
    return FFEA_GPU_OK;
}

int ffea_gpu_blob_get_connectivity(ffea_gpu_blob *b, int *ptr, int *es, long long *count) {
    if (!b) return FFEA_GPU_EINPUT;
    const HostModel &h = b->h;
    const int n = h.n_all, T = h.T;
    std::vector<int> cnt(n + 1, 0);
    for (int e = 0; e < T; ++e)
        for (int s = 0; s < 10; ++s) cnt[h.tets10[10 * (size_t)e + s] + 1]++;
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    if (count) *count = cnt[n];
    if (ptr) std::memcpy(ptr, cnt.data(), sizeof(int) * (n + 1));
    if (es) {
        std::vector<int> fill(n, 0);
        for (int e = 0; e < T; ++e)
            for (int s = 0; s < 10; ++s) {
                const int x = h.tets10[10 * (size_t)e + s];
                es[cnt[x] + fill[x]++] = 10 * e + s;
            }
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_blob_get_elements(ffea_gpu_blob *b, double *nf, double *vol, double *visc) {
    if (!b) return FFEA_GPU_EINPUT;
    return b->get_elements(nf, vol, visc);
}

int ffea_gpu_blob_get_rhs(ffea_gpu_blob *b, double *rhs) {
    if (!b || !rhs) return FFEA_GPU_EINPUT;
    return b->get_rhs(rhs);
}

int ffea_gpu_blob_solve_static(ffea_gpu_blob *b, const double *rhs, double *x, int *iterations) {
    if (!b || !rhs || !x) return FFEA_GPU_EINPUT;
    return b->solve_static(rhs, x, iterations);
}

int ffea_gpu_adjoint_create(ffea_gpu_blob *b, int window_steps, int checkpoint_every, ffea_gpu_adjoint **out) {
    if (!b || !out) return FFEA_GPU_EINPUT;
    *out = nullptr;
    if (b->adj_handle) {
        g_last_error = "this blob already has an adjoint";
        return FFEA_GPU_EINPUT;
    }
    int rc = b->adj_init(window_steps, checkpoint_every);
    if (rc) return rc;
    *out = new (std::nothrow) ffea_gpu_adjoint{b};
    if (!*out) {
        b->adj_release();
        return FFEA_GPU_ENOMEM;
    }
    b->adj_handle = *out;
    return FFEA_GPU_OK;
}

int ffea_gpu_adjoint_forward(ffea_gpu_adjoint *a, int *steps_done) {
    if (!a || !a->blob) return FFEA_GPU_EINPUT;
    return a->blob->adj_forward(steps_done);
}

int ffea_gpu_adjoint_backward(ffea_gpu_adjoint *a, const double *dl_dx_final, double *dl_dG, double *dl_dE,
                              double *dl_dA, double *dl_dB, double *dl_dx_initial) {
    if (!a || !a->blob || !dl_dx_final) return FFEA_GPU_EINPUT;
    return a->blob->adj_backward(dl_dx_final, dl_dG, dl_dE, dl_dA, dl_dB, dl_dx_initial);
}

void ffea_gpu_adjoint_destroy(ffea_gpu_adjoint *a) {
    if (!a) return;
    if (a->blob) {
        a->blob->adj_release();
        a->blob->adj_handle = nullptr;
    }
    delete a;
}

const char *ffea_gpu_last_error(void) { return g_last_error.c_str(); }

long long ffea_gpu_launch_count(void) { return ffea::launch_count(); }

}  // extern "C"
