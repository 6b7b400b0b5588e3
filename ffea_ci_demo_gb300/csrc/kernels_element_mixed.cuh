// kernels_element_mixed.cuh -- the mixed-precision element phase: node_prep_kernel and element_mixed_kernel.
//
// The reference's element loop (Blob::update_internal_forces, src/Blob.cpp:400-491, with
// tetra_element_linear's Jacobian, shape-function derivatives, stresses and force vector,
// src/tetra_element_linear.cpp:191-483) evaluated in FP32 except where FP32 cannot be trusted:
//
// * Geometry from displacements. node_prep_kernel writes each vertex's displacement from its rest
//   position, u = x - X (FP64 difference, rounded once to FP32), and its velocity in FP32. With
//   J0^-1 the rest-state inverse Jacobian (J_inv_0 of calc_rest_state_info, src/Blob.cpp:3080-3143) and
//   dU the edge matrix of the displacements, the current Jacobian is J = J0 (I + J0^-1 dU), so
//   K = I + J0^-1 dU is the reference's (J_inv_0 J), F = K^T its deformation gradient, det J = det J0 det K,
//   vol = vol_0 det K and J^-1 = K^-1 J0^-1. Everything is formed from Kd = K - I without forming K - I
//   by cancellation, and the stresses are rearranged the same way:
//     shear + bulk = (G / det K)(M + M^T + M M^T) + (E - 2G/3)(det K - 1)(det K + 1)/(2 det K) I,  M = F - I,
//   which is add_shear_elastic_stress + add_bulk_elastic_stress (:375-403) with the identity terms cancelled
//   exactly. No FP64 instruction runs for a well-shaped element.
// * Near-degenerate elements (det K <= 0.05: the element has lost 95 % of its rest volume, or inverted)
//   take the FP64 branch: J from the FP64 positions, cofactors, determinant and the inversion test
//   against last_det (the rest determinant: the mixed path does not update it, which is equivalent to the
//   reference's test against the previous step's determinant in every run that has not already stopped on
//   an inversion, since the sign never changes otherwise).
// * Viscous force of the inertial solvers: V_e v_e (get_element_velocity_vector + mat12_apply, :448-463)
//   equals vol sum_j dpsi_ja sigma_ij with sigma = B tr(L) I + A (L + L^T), L the velocity gradient
//   sum_b v_b (x) grad psi_b, so it is added to the stress before apply_stress_tensor (:436-443) instead of
//   forming the 12x12 matrix.
// * Noise: the element's 7 draws (add_fluctuating_stress, :412-431) start 7e draws after the step's stream
//   state; node_prep_kernel forms the state at the start of every 32-element chunk once per step and each
//   element makes one lane jump (A^(7 lane)). The stream states stay bit-exact; RAND(-.5,.5) is formed in
//   FP32 from the draw's integer, (k - (m1 + 1)/2)/(m1 + 1).
// * Staging and the deterministic block sum. A thread block of NT consecutive elements (EM_THREADS unless tuned)
//   loads the distinct vertices of its elements (listed on the host, at most 4 NT) into shared memory once;
//   each element reads its four nodes from there. The block then sums its elements' forces per vertex in
//   element order (the block's incidence list, sorted on the host) and writes one float4 per (block, vertex)
//   at the vertex's run of the node-major `parts` array, so the gather adds a vertex's block sums in block
//   order: the same result on every run, without float atomics.
#pragma once

#include "kernels.cuh"

namespace ffea {

// elements per thread block: the default, and the choices of the batch autotuner (multiples of the 32-element
// noise chunk)
constexpr int EM_THREADS = 128;
constexpr int EM_THREAD_CHOICES[3] = {64, 128, 256};
constexpr float EM_DEGENERATE = 0.05f;

// RAND(-.5,.5) of include/tetra_element_linear.h:119 in FP32. The MRG32k3a step is RngStream::U01's
// (src/RngStream.cpp:266-289) on integers; its value is k / (m1 + 1) with k = p1 - p2 (+ m1 when p1 <= p2)
// in [1, m1], so the draw less one half is (k - 2147483544) / 4294967088, an exact integer difference
// scaled once.
__device__ __forceinline__ float mrg_rand_half_f(uint32_t s[6]) {
    return (float)(int)(mrg_step(s) - 2147483544u) * (float)(1.0 / 4294967088.0);
}

struct NodePrepArgs {
    int N;
    const double *px, *py, *pz, *vx, *vy, *vz;
    const double *xr;              // 3 x N rest positions (SoA), the positions J_inv_0 was formed from
    float4 *u, *vf;                // out: displacement and (vf non-null) velocity in FP32
    int nchunks;                   // 0: no noise
    const uint32_t *rng_state;     // 6 per blob: its stream state at the start of the step
    const MrgJump *chunk_jump;     // A^(224 c), c = chunk index within the blob
    const int *chunk_blob;         // blob of each chunk (null: one blob)
    const int *chunk_off;          // first chunk of each blob (with chunk_blob)
    uint32_t *chunk_state;         // out: 6 per chunk
    int skip_nodes;                // 1: u and vf already hold this state (the fused mass-lumped gather wrote them)
};

// u = x - X and the velocities in FP32 for every vertex; the stream state at the start of every 32-element chunk
// (defined in engine_mixed.cu)
__global__ void __launch_bounds__(256) node_prep_kernel(NodePrepArgs g);

// The lane jumps A^(7 l), l < 32, in shared memory: 18 words each, padded to 20 so that a quarter warp's 16-byte
// loads of eight different lanes' jumps fall in distinct banks.
constexpr int EM_JUMP_WORDS = 20;

// asynchronous global -> shared copies (cp.async, completed by cp_async_wait_all): a block's staging loads are all
// in flight at once without holding registers
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void stage_lane_jumps(const MrgJump *lane_jump, uint32_t *s_jump, int tid, int nt) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(lane_jump);
    for (int i = tid; i < 32 * 18; i += nt) cp_async4(s_jump + EM_JUMP_WORDS * (i / 18) + i % 18, src + i);
}

// the elements' forces in shared memory, EM_F_STRIDE floats apart: 13 is coprime to the 32 banks, so a warp's
// stores of its 32 elements' k-th force component hit 32 different banks
constexpr int EM_F_STRIDE = 13;
static_assert(EM_F_STRIDE >= 12 && EM_F_STRIDE <= 16, "the forces overlay the 4 NT staged float4 displacements");

// per-element inputs staged by element_mixed_kernel, EM_EL_ROWS rows of one float per element of the block:
// J0^-1 (9, row-major), vol0, G, E, A, B
constexpr int EM_EL_ROWS = 14;

// bytes of dynamic shared memory of an element_mixed_kernel block of nt elements
__host__ __device__ __forceinline__ int em_smem_bytes(int nt, bool inertial, bool noise) {
    return (inertial ? 8 : 4) * nt * 16 + EM_EL_ROWS * nt * 4 + 4 * nt * 2 + (noise ? 32 * EM_JUMP_WORDS * 4 : 0);
}

// Element e's 7 draws of add_fluctuating_stress less one half (RAND(-.5,.5)), in draw order. They start 7 le draws
// after its blob's state at the start of the step (le the element's index in its blob): from the state at the
// start of its 32-element chunk (node_prep_kernel) by one jump of A^(7 (le mod 32)) (staged by stage_lane_jumps).
// (element_chunk_state loads the chunk's state; element_draws makes the draws from it)
__device__ __forceinline__ int element_chunk_state(const ElemArgs<float> &g, int e, uint32_t (&base)[6]) {
    int le = e, chunk = e >> 5;
    if (g.elem_blob) {
        const int b = g.elem_blob[e];
        le = e - g.elem_off[b];
        chunk = g.chunk_off[b] + (le >> 5);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) base[k] = g.chunk_state[6 * (size_t)chunk + k];
    return le;
}

__device__ __forceinline__ void element_draws(const uint32_t (&base)[6], int le, const uint32_t *s_jump,
                                              float (&rn)[7]) {
    uint32_t s6[6];
    MrgJump J;
    const uint4 *q = reinterpret_cast<const uint4 *>(s_jump + EM_JUMP_WORDS * (le & 31));
    uint32_t w[20];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint4 v = q[k];
        w[4 * k] = v.x; w[4 * k + 1] = v.y; w[4 * k + 2] = v.z; w[4 * k + 3] = v.w;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        J.a[k] = w[k];
        J.b[k] = w[9 + k];
    }
    mrg_apply(J, base, s6);
#pragma unroll
    for (int k = 0; k < 7; ++k) rn[k] = mrg_rand_half_f(s6);
}

// The FP64 Jacobian of calculate_jacobian / calc_shape_function_derivatives_and_volume
// (src/tetra_element_linear.cpp:191-292) for a near-degenerate or inverted element, out of line so that the
// common FP32 path keeps its registers: dpsi, volume, det K, delta = det K - 1 and M = (J0^-1 J)^T - I, or ok = false
// (with the inversion flags raised) for an inverted element.
struct ElemFp64 {
    float dpsi[12], M[9];
    float vol, dK, delta;
    int ok;
};

static __device__ __noinline__ ElemFp64 element_fp64_jacobian(const ElemArgs<float> &g, int e) {
    ElemFp64 o;
    const int4 t = g.tet[e];
    const double x0 = g.px[t.x], y0 = g.py[t.x], z0 = g.pz[t.x];
    double J[3][3];
    J[0][0] = g.px[t.y] - x0; J[0][1] = g.py[t.y] - y0; J[0][2] = g.pz[t.y] - z0;
    J[1][0] = g.px[t.z] - x0; J[1][1] = g.py[t.z] - y0; J[1][2] = g.pz[t.z] - z0;
    J[2][0] = g.px[t.w] - x0; J[2][1] = g.py[t.w] - y0; J[2][2] = g.pz[t.w] - z0;
    double d[12];
    d[1] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    d[2] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    d[3] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    d[5] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
    d[6] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
    d[7] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
    d[9] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
    d[10] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
    d[11] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
    const double det = J[0][0] * d[1] + J[1][0] * d[2] + J[2][0] * d[3];
    const double last = g.recompute ? det : g.last_det[e];
    if (last * det < 0) {
        atomicAdd(&g.st->inversions, 1);
        atomicExch(&g.st->abort, 1);
        o.ok = 0;
        return o;
    }
    o.ok = 1;
    const double vold = (1.0 / 6.0) * fabs(det);
    const double idet = 1.0 / det;
#pragma unroll
    for (int k = 0; k < 12; ++k)
        if (k & 3) o.dpsi[k] = (float)(d[k] * idet);
    o.dpsi[0] = -(o.dpsi[1] + o.dpsi[2] + o.dpsi[3]);
    o.dpsi[4] = -(o.dpsi[5] + o.dpsi[6] + o.dpsi[7]);
    o.dpsi[8] = -(o.dpsi[9] + o.dpsi[10] + o.dpsi[11]);
    o.vol = (float)vold;
    const size_t T = g.T;
    o.dK = (float)(vold / (double)g.vol0[e]);
    o.delta = o.dK - 1.f;
    // M = (J0^-1 J)^T - I from the FP64 Jacobian
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const double j0 = g.jinv[3 * r * T + e], j1 = g.jinv[(3 * r + 1) * T + e], j2 = g.jinv[(3 * r + 2) * T + e];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            o.M[3 * c + r] = (float)(j0 * J[0][c] + j1 * J[1][c] + j2 * J[2][c] - (r == c ? 1.0 : 0.0));
    }
    return o;
}

// One element's forces (f[3a + c]: node a, component c; FORCES), shape-function derivatives and volume, with the
// viscous stress of the nodes' velocities vn when `visc` and the thermal stress of the draws rn (element_draws)
// when noise is on; returns false (and raises the inversion flags) for an inverted element.
// sel: the element's staged inputs (EM_EL_ROWS rows, `stride` apart).
template <bool FORCES>
__device__ __forceinline__ bool element_mixed_eval(const ElemArgs<float> &g, int e, const float *sel, int stride,
                                                   const float4 (&un)[4], bool visc, const float4 (&vn)[4],
                                                   const float (&rn)[7], float (&f)[12], float (&dpsi)[12],
                                                   float &vol) {
    float Ji[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Ji[k] = sel[k * stride];
    const float vol0 = sel[9 * stride];
    // Kd = J0^-1 dU, dU rows = edge displacements u_1 - u_0, u_2 - u_0, u_3 - u_0
    float dU[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        dU[r][0] = un[r + 1].x - un[0].x;
        dU[r][1] = un[r + 1].y - un[0].y;
        dU[r][2] = un[r + 1].z - un[0].z;
    }
    float Kd[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Kd[r][c] = Ji[3 * r] * dU[0][c] + Ji[3 * r + 1] * dU[1][c] + Ji[3 * r + 2] * dU[2][c];
    // det(I + Kd) - 1 = tr Kd + (principal 2x2 minors) + det Kd
    const float minors = (Kd[0][0] * Kd[1][1] - Kd[0][1] * Kd[1][0]) + (Kd[0][0] * Kd[2][2] - Kd[0][2] * Kd[2][0]) +
                         (Kd[1][1] * Kd[2][2] - Kd[1][2] * Kd[2][1]);
    const float detKd = Kd[0][0] * (Kd[1][1] * Kd[2][2] - Kd[1][2] * Kd[2][1]) -
                        Kd[0][1] * (Kd[1][0] * Kd[2][2] - Kd[1][2] * Kd[2][0]) +
                        Kd[0][2] * (Kd[1][0] * Kd[2][1] - Kd[1][1] * Kd[2][0]);
    float delta = (Kd[0][0] + Kd[1][1] + Kd[2][2]) + minors + detKd;
    float dK = 1.f + delta, id;
    float M[3][3];  // F - I = Kd^T
    if (dK > EM_DEGENERATE) {
        // K^-1 = adj(K) / det K, then J^-1 = K^-1 J0^-1: dpsi[4j + a] = (J^-1)[j][a - 1]
        const float k00 = 1.f + Kd[0][0], k11 = 1.f + Kd[1][1], k22 = 1.f + Kd[2][2];
        id = __frcp_rn(dK);  // 1 / det K, correctly rounded (the division's value)
        float Ki[3][3];
        Ki[0][0] = (k11 * k22 - Kd[1][2] * Kd[2][1]) * id;
        Ki[0][1] = (Kd[0][2] * Kd[2][1] - Kd[0][1] * k22) * id;
        Ki[0][2] = (Kd[0][1] * Kd[1][2] - Kd[0][2] * k11) * id;
        Ki[1][0] = (Kd[1][2] * Kd[2][0] - Kd[1][0] * k22) * id;
        Ki[1][1] = (k00 * k22 - Kd[0][2] * Kd[2][0]) * id;
        Ki[1][2] = (Kd[0][2] * Kd[1][0] - k00 * Kd[1][2]) * id;
        Ki[2][0] = (Kd[1][0] * Kd[2][1] - k11 * Kd[2][0]) * id;
        Ki[2][1] = (Kd[0][1] * Kd[2][0] - k00 * Kd[2][1]) * id;
        Ki[2][2] = (k00 * k11 - Kd[0][1] * Kd[1][0]) * id;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
#pragma unroll
            for (int m = 0; m < 3; ++m)
                dpsi[4 * j + m + 1] = Ki[j][0] * Ji[m] + Ki[j][1] * Ji[3 + m] + Ki[j][2] * Ji[6 + m];
            dpsi[4 * j] = -(dpsi[4 * j + 1] + dpsi[4 * j + 2] + dpsi[4 * j + 3]);
        }
        vol = vol0 * dK;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) M[i][j] = Kd[j][i];
    } else {
        // near-degenerate or inverted
        const ElemFp64 o = element_fp64_jacobian(g, e);
        if (!o.ok) return false;
#pragma unroll
        for (int k = 0; k < 12; ++k) dpsi[k] = o.dpsi[k];
        vol = o.vol;
        dK = o.dK;
        delta = o.delta;
        id = 1.f / dK;
#pragma unroll
        for (int k = 0; k < 9; ++k) M[k / 3][k % 3] = o.M[k];
    }
    if (!FORCES) return true;
    const float G = sel[10 * stride], E = sel[11 * stride], A = sel[12 * stride], B = sel[13 * stride];
    // elastic stress: (G / det K)(M + M^T + M M^T) + (E - 2G/3) delta (2 + delta) / (2 det K) I
    float S[3][3];
    {
        const float gk = G * id;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                const float s = gk * (M[i][j] + M[j][i] + (M[i][0] * M[j][0] + M[i][1] * M[j][1] + M[i][2] * M[j][2]));
                S[i][j] = s;
                S[j][i] = s;
            }
        const float c2 = E - G * 2.f / 3.f;
        const float cb = 0.5f * c2 * delta * (2.f + delta) * id;
        S[0][0] += cb;
        S[1][1] += cb;
        S[2][2] += cb;
    }
    // add_fluctuating_stress :412-431 (draws b, d0, d1, d2, o01, o02, o12)
    if (g.calc_noise == 1) {
        // sqrt(24 kT / (vol dt)) as sqrt(24 kT / dt) / sqrt(vol), and sqrt(2A) as sqrt(2) sqrt(A): the noise
        // amplitude to a few FP32 ulp with one correctly rounded square root fewer and no division
        const float c = sqrtf((24.f * g.kT) / g.dt) * rsqrtf(vol);
        const float bf = sqrtf(B) * rn[0];
        const float a1 = sqrtf(A), a2 = 1.41421356f * a1;
        S[0][0] += c * (a2 * rn[1] + bf);
        S[1][1] += c * (a2 * rn[2] + bf);
        S[2][2] += c * (a2 * rn[3] + bf);
        const float o01 = c * a1 * rn[4];
        const float o02 = c * a1 * rn[5];
        const float o12 = c * a1 * rn[6];
        S[0][1] += o01; S[1][0] += o01;
        S[0][2] += o02; S[2][0] += o02;
        S[1][2] += o12; S[2][1] += o12;
    }
    // viscous stress of the inertial solvers from the velocity gradient L[i][j] = sum_b v_b[i] dpsi[4j + b]
    if (visc) {
        float L[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            L[0][j] = vn[0].x * dpsi[4 * j] + vn[1].x * dpsi[4 * j + 1] + vn[2].x * dpsi[4 * j + 2] + vn[3].x * dpsi[4 * j + 3];
            L[1][j] = vn[0].y * dpsi[4 * j] + vn[1].y * dpsi[4 * j + 1] + vn[2].y * dpsi[4 * j + 2] + vn[3].y * dpsi[4 * j + 3];
            L[2][j] = vn[0].z * dpsi[4 * j] + vn[1].z * dpsi[4 * j + 1] + vn[2].z * dpsi[4 * j + 2] + vn[3].z * dpsi[4 * j + 3];
        }
        const float btr = B * (L[0][0] + L[1][1] + L[2][2]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) S[i][j] += A * (L[i][j] + L[j][i]) + (i == j ? btr : 0.f);
    }
    // apply_stress_tensor :436-443 and add_element_force_vector :468-483 (node_force = -du)
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            f[3 * a + i] = -(vol * (dpsi[a] * S[i][0] + dpsi[4 + a] * S[i][1] + dpsi[8 + a] * S[i][2]));
    return true;
}

// PARTIALS: block sums per vertex into g.parts (the step); else per-element forces into g.ef when it is set (or
// none: recompute for the assembly's geometry only). g.geom, when set, gets dpsi and vol for the assembly.
template <bool PARTIALS, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) element_mixed_kernel(ElemArgs<float> g) {
    // dynamic shared memory (em_smem_bytes): staged displacements (4 NT; then the elements' forces, 12 per
    // element), velocities (4 NT, inertial solvers), the elements' inputs (EM_EL_ROWS x NT), the block's incidence
    // list (4 NT codes), the lane jumps (noise)
    extern __shared__ __align__(16) float4 em_smem[];
    __shared__ int s_abort;
    const int tid = threadIdx.x, blk = blockIdx.x;
    const bool inertial = !g.nomass;
    const bool forces = PARTIALS || g.ef != nullptr;
    const bool noise = forces && g.calc_noise == 1;
    float4 *s_u = em_smem, *s_v = em_smem + 4 * NT;
    float *s_el = reinterpret_cast<float *>(em_smem + (inertial ? 8 : 4) * NT);
    unsigned short *s_il = reinterpret_cast<unsigned short *>(s_el + EM_EL_ROWS * NT);
    uint32_t *s_jump = reinterpret_cast<uint32_t *>(s_il + 4 * NT);
    if (tid == 0) s_abort = g.st->abort;
    if (noise) stage_lane_jumps(g.lane_jump, s_jump, tid, NT);
    const int n0 = g.cta_ptr[blk], nn = g.cta_ptr[blk + 1] - n0;
    for (int i = tid; i < nn; i += NT) {
        const int node = g.cta_nodes[n0 + i];
        cp_async16(s_u + i, g.u + node);
        if (inertial) cp_async16(s_v + i, g.vf + node);
    }
    if (PARTIALS) {  // 4 NT codes = NT / 2 chunks of 16 bytes, 16-byte aligned (4 NT 2 bytes per block)
        const uint4 *src = reinterpret_cast<const uint4 *>(g.inc_local + 4 * NT * (size_t)blk);
        for (int i = tid; i < NT / 2; i += NT) cp_async16(reinterpret_cast<uint4 *>(s_il) + i, src + i);
    }
    const int e = blk * NT + tid;
    const bool live = e < g.T;
    if (live) {
        const size_t T = g.T;
#pragma unroll
        for (int k = 0; k < 9; ++k) cp_async4(s_el + k * NT + tid, g.jinv + k * T + e);
        cp_async4(s_el + 9 * NT + tid, g.vol0 + e);
        if (forces) {
            cp_async4(s_el + 10 * NT + tid, g.G + e);
            cp_async4(s_el + 11 * NT + tid, g.E + e);
            cp_async4(s_el + 12 * NT + tid, g.A + e);
            cp_async4(s_el + 13 * NT + tid, g.B + e);
        }
    }
    const ushort4 l = live ? g.loc[e] : make_ushort4(0, 0, 0, 0);
    uint32_t base[6];
    int le = 0;
    if (noise && live) le = element_chunk_state(g, e, base);
    cp_async_wait_all();
    __syncthreads();
    if (s_abort) return;  // uniform: read from shared memory after the barrier
    // the draws first, while little else is held in registers
    float rn[7];
    if (noise && live) element_draws(base, le, s_jump, rn);
    float f[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) f[k] = 0.f;
    if (live) {
        const float4 un[4] = {s_u[l.x], s_u[l.y], s_u[l.z], s_u[l.w]};
        float4 vb[4] = {};
        if (inertial) {
            vb[0] = s_v[l.x]; vb[1] = s_v[l.y]; vb[2] = s_v[l.z]; vb[3] = s_v[l.w];
        }
        float dpsi[12], vol;
        const bool ok = forces ? element_mixed_eval<true>(g, e, s_el + tid, NT, un, inertial, vb, rn, f, dpsi, vol)
                               : element_mixed_eval<false>(g, e, s_el + tid, NT, un, false, vb, rn, f, dpsi, vol);
        if (!ok) {
#pragma unroll
            for (int k = 0; k < 12; ++k) f[k] = 0.f;  // inverted: the step is void; contribute nothing
        } else {
            if (g.geom) {
                float4 *gm = reinterpret_cast<float4 *>(g.geom + 16 * (size_t)e);
                gm[0] = make_float4(dpsi[0], dpsi[1], dpsi[2], dpsi[3]);
                gm[1] = make_float4(dpsi[4], dpsi[5], dpsi[6], dpsi[7]);
                gm[2] = make_float4(dpsi[8], dpsi[9], dpsi[10], dpsi[11]);
                gm[3] = make_float4(vol, 0.f, 0.f, 0.f);
            }
            if (!PARTIALS && g.ef) {
                float *ef = g.ef + 12 * (size_t)e;
#pragma unroll
                for (int k = 0; k < 12; ++k) ef[k] = f[k];
            }
        }
    }
    if constexpr (!PARTIALS) return;
    __syncthreads();  // every element has read its nodes: the staging area now takes the forces
    float *s_f = reinterpret_cast<float *>(s_u);
#pragma unroll
    for (int k = 0; k < 12; ++k) s_f[tid * EM_F_STRIDE + k] = f[k];
    __syncthreads();
    // each vertex of the block: its elements' forces in element order, from the block's incidence list
    // (code 4 el + slot: the force sits at s_f[EM_F_STRIDE el + 3 slot])
    const int ne = min(NT, g.T - blk * NT);
    const unsigned short *il = s_il;
    for (int i = tid; i < nn; i += NT) {
        const int m0 = g.inc_start[n0 + i], m1 = (i + 1 < nn) ? (int)g.inc_start[n0 + i + 1] : 4 * ne;
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        for (int m = m0; m < m1; ++m) {
            const int code = il[m];
            const float *c = s_f + EM_F_STRIDE * (code >> 2) + 3 * (code & 3);
            a0 += c[0];
            a1 += c[1];
            a2 += c[2];
        }
        g.parts[g.perm[n0 + i]] = make_float4(a0, a1, a2, 0.f);
    }
}

}  // namespace ffea
