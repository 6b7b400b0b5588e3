// kernels.cuh -- the blob-step kernels, templated on the arithmetic type R.
//
// R = double is the plain FP64 path. Its translation unit is compiled with
// -fmad=false, and every expression below is written in the reference's
// evaluation order, so the element forces, viscosity matrices, assembled
// matrix values, right-hand sides and SpMV rows are bit-identical to the
// reference's (src/tetra_element_linear.cpp, src/Blob.cpp,
// src/SparseMatrixFixedPattern.cpp); only the CG's cross-node reductions are
// summed in a different (fixed) order.
//
// R = float is the mixed path: stress, noise scaling, matrix values, SpMV and
// CG vectors are FP32; dot products and norms are accumulated across nodes in
// FP64; positions are FP64 accumulators. Its element phase is
// element_mixed_kernel (kernels_element_mixed.cuh), which keeps the Jacobian
// in FP64 only for near-degenerate elements; element_kernel below is the FP64
// path's.
//
// Layouts (N vertex nodes, T elements):
//   positions/velocities   SoA double px,py,pz / vx,vy,vz
//   element data           SoA by field (coalesced per element)
//   element outputs        ef[12*e + 3*a + c] (node a of element e, component c), geom[16*e + k]
//   CG vectors             padded AoS, 4 per node: v[4*a + c]
//   matrix                 3x3 blocks in SELL-32: slice s = 32 consecutive rows, slot(k,lane) =
//                          slice_ptr[s] + 32*k + lane; block values val[9*slice_ptr[s] + 32*(9*k + c) + lane]
#pragma once

#include "common.cuh"

namespace ffea {

// ---------------------------------------------------------------------------
// element kernel
// ---------------------------------------------------------------------------
template <class R>
struct ElemArgs {
    int T, nomass, calc_noise;
    R kT, dt;
    const int4 *tet;
    const double *px, *py, *pz;
    const double *vx, *vy, *vz;
    const R *jinv;                 // 9*T, SoA jinv[k*T + e]
    const R *G, *E, *A, *B, *vol0; // per element
    double *last_det;
    R *ef;    // 12*T
    R *geom;  // 16*T: dpsi[12], vol
    const uint32_t *rng_state;     // 6 per stream: stream state at the start of the step
    const int *elem_blob;          // batch: blob of each element (null for one blob)
    const int *elem_off;           // batch: first element of each blob
    const MrgJump *chunk_jump;     // ceil(T/32): A^(7*32*c)
    const MrgJump *lane_jump;      // 32: A^(7*l)
    int recompute;                 // 1: re-evaluation at stored positions (no inversion test, last_det kept)
    DevStatus *st;
    // mixed path (element_mixed_kernel): node displacements and velocities in FP32 (node_prep_kernel), the thread
    // blocks' vertex lists, each element's vertices as indices into its block's list, the node-major block sums
    // and their positions, and the stream state at every 32-element chunk
    const float4 *u, *vf;
    const int *cta_ptr, *cta_nodes;
    const ushort4 *loc;
    const unsigned short *inc_local, *inc_start;  // each block's incidence, by vertex then element
    float4 *parts;
    const int *perm;
    const uint32_t *chunk_state;   // 6 per 32-element chunk: the stream state at the chunk's first draw
    const int *chunk_off;          // batch: first chunk of each blob
    int em_threads;                // elements per thread block, as the block lists were built (0: EM_THREADS)
};

// V[r][c] of tetra_element_linear::create_viscosity_matrix (src/tetra_element_linear.cpp:298-327)
// for r = a + 4i, c = b + 4j, evaluated exactly as the reference builds the entry it mirrors.
template <class R>
__device__ __forceinline__ R visc_entry(const R *dpsi, R A, R B, R vol, int r, int c) {
    if (r > c) { int t = r; r = c; c = t; }
    const int i = r >> 2, a = r & 3, j = c >> 2, b = c & 3;
    if (i == j) {
        const R t = dpsi[4 * i + a] * dpsi[4 * i + b] * (A + B);
        const R d2 = (dpsi[a] * dpsi[b] + dpsi[4 + a] * dpsi[4 + b] + dpsi[8 + a] * dpsi[8 + b]);
        return (t + d2 * A) * vol;
    }
    if (a == b) return ((B + A) * (dpsi[4 * i + a] * dpsi[4 * j + a])) * vol;
    return (B * (dpsi[4 * i + a] * dpsi[4 * j + b]) + A * (dpsi[4 * i + b] * dpsi[4 * j + a])) * vol;
}

template <class R>
__global__ void __launch_bounds__(128) element_kernel(ElemArgs<R> g) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.T || g.st->abort) return;
    const int4 t = g.tet[e];
    // calculate_jacobian :191-203 (FP64 in both paths)
    const double x0 = g.px[t.x], y0 = g.py[t.x], z0 = g.pz[t.x];
    double J[3][3];
    J[0][0] = g.px[t.y] - x0; J[0][1] = g.py[t.y] - y0; J[0][2] = g.pz[t.y] - z0;
    J[1][0] = g.px[t.z] - x0; J[1][1] = g.py[t.z] - y0; J[1][2] = g.pz[t.z] - z0;
    J[2][0] = g.px[t.w] - x0; J[2][1] = g.py[t.w] - y0; J[2][2] = g.pz[t.w] - z0;
    // calc_shape_function_derivatives_and_volume :222-292 (FP64 in both paths)
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
    double det = J[0][0] * d[1] + J[1][0] * d[2] + J[2][0] * d[3];
    const double last = g.recompute ? det : g.last_det[e];
    double vold;
    if (last * det < 0) {
        // inverted: the reference returns before updating vol and dividing dpsi; the step is void
        atomicAdd(&g.st->inversions, 1);
        atomicExch(&g.st->abort, 1);
        return;
    }
    if (!g.recompute) g.last_det[e] = det;
    vold = (1.0 / 6.0) * fabs(det);
    det = 1.0 / det;
    d[1] *= det; d[2] *= det; d[3] *= det;
    d[5] *= det; d[6] *= det; d[7] *= det;
    d[9] *= det; d[10] *= det; d[11] *= det;
    d[0] = -(d[1] + d[2] + d[3]);
    d[4] = -(d[5] + d[6] + d[7]);
    d[8] = -(d[9] + d[10] + d[11]);
    R dpsi[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) dpsi[k] = (R)d[k];
    const R vol = (R)vold;
    R Jr[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Jr[i][j] = (R)J[i][j];
    const R G = g.G[e], E = g.E[e], A = g.A[e], B = g.B[e], vol0 = g.vol0[e];
    // add_shear_elastic_stress :375-392
    R Ji[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Ji[k] = g.jinv[(size_t)k * g.T + e];
    R F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            R s = 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) s += Jr[k][i] * Ji[3 * j + k];
            F[i][j] = s;
        }
    R S[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            R s = 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) s += F[i][k] * F[j][k];
            S[i][j] = s;
        }
    const R sc = (G * vol0 / vol);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[i][j] *= sc;
    S[0][0] -= G;
    S[1][1] -= G;
    S[2][2] -= G;
    // add_bulk_elastic_stress :397-403
    {
        const R c_2 = E - G * (R)2.0 / (R)3.0;
        const R c = G * ((R)1.0 - (vol0 / vol)) + (R)0.5 * c_2 * ((vol / vol0) - (vol0 / vol));
        S[0][0] += c;
        S[1][1] += c;
        S[2][2] += c;
    }
    // add_fluctuating_stress :412-431, draws in the single-thread reference order
    if (g.calc_noise == 1) {
        // element e of a blob starts 7e draws after the blob's stream state
        uint32_t base[6], s6[6];
        int le = e;
        const uint32_t *rs = g.rng_state;
        if (g.elem_blob) {
            const int b = g.elem_blob[e];
            le = e - g.elem_off[b];
            rs += 6 * (size_t)b;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) s6[k] = rs[k];
        mrg_apply(g.chunk_jump[le >> 5], s6, base);
        mrg_apply(g.lane_jump[le & 31], base, s6);
        const R c = sqrt(((R)24 * g.kT) / (vol * g.dt));
        const R bf = sqrt(B) * (R)mrg_rand_half(s6);
        S[0][0] += c * (sqrt((R)2 * A) * (R)mrg_rand_half(s6) + bf);
        S[1][1] += c * (sqrt((R)2 * A) * (R)mrg_rand_half(s6) + bf);
        S[2][2] += c * (sqrt((R)2 * A) * (R)mrg_rand_half(s6) + bf);
        S[0][1] += c * sqrt(A) * (R)mrg_rand_half(s6);
        S[0][2] += c * sqrt(A) * (R)mrg_rand_half(s6);
        S[1][2] += c * sqrt(A) * (R)mrg_rand_half(s6);
        S[1][0] = S[0][1];
        S[2][0] = S[0][2];
        S[2][1] = S[1][2];
    }
    R du[12];
    if (!g.nomass) {
        // get_element_velocity_vector :448-463 + mat12_apply (src/mat_vec_fns.cpp:28-36)
        const int nd[4] = {t.x, t.y, t.z, t.w};
        R v[12];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            v[a] = (R)g.vx[nd[a]];
            v[4 + a] = (R)g.vy[nd[a]];
            v[8 + a] = (R)g.vz[nd[a]];
        }
#pragma unroll
        for (int i = 0; i < 12; ++i) {
            R s = 0;
#pragma unroll
            for (int j = 0; j < 12; ++j) s += visc_entry<R>(dpsi, A, B, vol, i, j) * v[j];
            du[i] = s;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 12; ++i) du[i] = 0;
    }
    // apply_stress_tensor :436-443
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        du[4 * i] += vol * (dpsi[0] * S[i][0] + dpsi[4] * S[i][1] + dpsi[8] * S[i][2]);
        du[4 * i + 1] += vol * (dpsi[1] * S[i][0] + dpsi[5] * S[i][1] + dpsi[9] * S[i][2]);
        du[4 * i + 2] += vol * (dpsi[2] * S[i][0] + dpsi[6] * S[i][1] + dpsi[10] * S[i][2]);
        du[4 * i + 3] += vol * (dpsi[3] * S[i][0] + dpsi[7] * S[i][1] + dpsi[11] * S[i][2]);
    }
    // add_element_force_vector :468-483 (node_force starts at zero every step)
    R *ef = g.ef + 12 * (size_t)e;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) ef[3 * a + c] = (R)0 - du[4 * c + a];
    R *gm = g.geom + 16 * (size_t)e;
#pragma unroll
    for (int k = 0; k < 12; ++k) gm[k] = dpsi[k];
    gm[12] = vol;
}

// ---------------------------------------------------------------------------
// matrix assembly: CSR values = sum of element sources in element order
// (SparseMatrixFixedPattern::build + sparse_entry_sources::sum_all_sources)
// ---------------------------------------------------------------------------
template <class R>
struct AsmArgs {
    int N;
    long long nslots;       // 32 x the slices' widths
    const int *grp_slice;   // slice of each group of 32 slots
    const int *slice_ptr, *rowlen, *bcol, *diagk;
    const int *src_ptr;
    const unsigned *src;    // (element << 4) | (slot_a << 2) | slot_b ; 0xffffffff = identity
    const R *geom, *A, *B;  // per element
    const double *drag;     // per node or null
    R *val;
    R *dinv;                // 4*N
    R *diag;                // 4*N diagonal of V (mixed path) or null
    DevStatus *st;
    int threads;            // threads per block (0: the default); 64, 128 or 256
    int split;              // 0: three threads per slot while they fit on the GPU at once; 1: three; 2: one
};

constexpr unsigned SRC_IDENTITY = 0xffffffffu;

// The slot's sources are summed from zero in registration order, so each FP64 value rounds as
// sum_all_sources' does; the diagonal slot of a row also gives the Jacobi inverse. Padding slots past a row's
// length are never read and are skipped.
// SPLIT = false: one thread per matrix slot (3x3 block), which reads each source's element geometry once.
// SPLIT = true: three threads per slot, one per block row (a warp takes one block row of 32 consecutive slots
// of a slice), for matrices too small to fill the GPU, where the length of each thread's FP64 chain sets the
// time rather than the geometry reads.
template <class R>
__device__ __forceinline__ R sel3(const R (&x)[3], int i) {
    return i == 0 ? x[0] : (i == 1 ? x[1] : x[2]);
}

// visc_entry for the 3x3 block of element nodes (a, b) from their gradients ga = grad psi_a, gb = grad psi_b:
// entry (i, j) of the block is V[a + 4i][b + 4j]. Each case of visc_entry is symmetric under its mirror
// (a, i) <-> (b, j) (products commute exactly), so the entry needs no swap and equals visc_entry's bit for bit.
template <class R>
__device__ __forceinline__ R visc_block_entry(const R (&ga)[3], const R (&gb)[3], bool same, R A, R B, R vol, int i,
                                              int j) {
    if (i == j) {
        const R t = sel3(ga, i) * sel3(gb, i) * (A + B);
        const R d2 = (ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2]);
        return (t + d2 * A) * vol;
    }
    if (same) return ((B + A) * (sel3(ga, i) * sel3(ga, j))) * vol;
    return (B * (sel3(ga, i) * sel3(gb, j)) + A * (sel3(gb, i) * sel3(ga, j))) * vol;
}

// One assembly source: the gradients of its two element nodes, the element's volume and viscosity coefficients
// (nothing for the identity source of a pinned row).
template <class R>
__device__ __forceinline__ void asm_load(const AsmArgs<R> &g, unsigned code, R (&ga)[3], R (&gb)[3], R (&vab)[3]) {
    if (code == SRC_IDENTITY) return;
    const int e = (int)(code >> 4), pa = (code >> 2) & 3, pb = code & 3;
    const R *gm = g.geom + 16 * (size_t)e;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ga[c] = gm[4 * c + pa];
        gb[c] = gm[4 * c + pb];
    }
    vab[0] = gm[12];
    vab[1] = g.A[e];
    vab[2] = g.B[e];
}

// ... added to the thread's NB block rows (from block row b0) of the slot, entries in row-major order
template <class R, int NB>
__device__ __forceinline__ void asm_add(R (&v)[3 * NB], unsigned code, const R (&ga)[3], const R (&gb)[3],
                                        const R (&vab)[3], int b0) {
    if (code == SRC_IDENTITY) {
#pragma unroll
        for (int i = 0; i < NB; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                if (j == b0 + i) v[3 * i + j] += (R)1;
        return;
    }
    const bool same = ((code >> 2) & 3) == (code & 3);
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[3 * i + j] += visc_block_entry<R>(ga, gb, same, vab[1], vab[2], vab[0], b0 + i, j);
}

template <class R, bool SPLIT>
__global__ void __launch_bounds__(256) assemble_kernel(AsmArgs<R> g) {
    constexpr int NB = SPLIT ? 1 : 3;  // block rows per thread
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long slot = SPLIT ? ((t >> 5) / 3) * 32 + (t & 31) : t;
    const int b0 = SPLIT ? (int)((t >> 5) % 3) : 0;  // first block row
    if (slot >= g.nslots || g.st->abort) return;
    const int s = g.grp_slice[slot >> 5];
    const int lane = (int)(slot & 31);
    const int a = 32 * s + lane;
    if (a >= g.N) return;
    const int k = (int)((slot >> 5) - (g.slice_ptr[s] >> 5));
    if (k >= g.rowlen[a]) return;
    R v[3 * NB];
#pragma unroll
    for (int c = 0; c < 3 * NB; ++c) v[c] = (R)0.0;
    // two sources per trip: both sources' loads issue before either is summed (the sums keep registration order)
    const int q1 = g.src_ptr[slot + 1];
    int q = g.src_ptr[slot];
    for (; q + 1 < q1; q += 2) {
        const unsigned c0 = g.src[q], c1 = g.src[q + 1];
        R a0[3], e0[3], w0[3], a1[3], e1[3], w1[3];
        asm_load(g, c0, a0, e0, w0);
        asm_load(g, c1, a1, e1, w1);
        asm_add<R, NB>(v, c0, a0, e0, w0, b0);
        asm_add<R, NB>(v, c1, a1, e1, w1, b0);
    }
    if (q < q1) {
        const unsigned c0 = g.src[q];
        R a0[3], e0[3], w0[3];
        asm_load(g, c0, a0, e0, w0);
        asm_add<R, NB>(v, c0, a0, e0, w0, b0);
    }
    if (k == g.diagk[a]) {
#pragma unroll
        for (int i = 0; i < NB; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                if (j != b0 + i) continue;
                R &d = v[3 * i + j];
                if (g.drag) d += (R)g.drag[a];
                // calc_inverse_diagonal (src/SparseMatrixFixedPattern.cpp:305-312)
                g.dinv[4 * a + j] = (R)1.0 / d;
                if (g.diag) g.diag[4 * a + j] = d;
            }
    }
    R *vp = g.val + 9 * (size_t)g.slice_ptr[s] + 32 * 9 * (size_t)k + lane + 32 * 3 * b0;
#pragma unroll
    for (int c = 0; c < 3 * NB; ++c) vp[32 * c] = v[c];
}

// ---------------------------------------------------------------------------
// force gather (Blob::aggregate_forces_and_solve :3152-3158) + solver set-up
// ---------------------------------------------------------------------------
// Forces on nodes other than the elements' (Blob::apply_ctforces, src/Blob.cpp:1676-1743; the Stokes part of
// aggregate_forces_and_solve, :3172-3224; linearise_force, :781-799), on the reference numbering:
// constant linear forces (before the element contributions), constant surface forces (after them, face by face),
// Stokes noise (3 draws per node after the elements' 7T), and the move of midpoint forces to their edge ends.
struct NodeForces {
    int on;                        // any of the below
    int noise;                     // Stokes noise
    double kT, dt;
    const uint32_t *rng_state;     // the step's stream state
    const MrgJump *chunk_jump;     // A^(base + 96 c): first draw of node chunk c (reference numbering)
    const MrgJump *lane_jump;      // A^(3 l)
    const int *node_orig;          // vertex -> reference node index
    const double *node_drag;       // vertex Stokes drag
    const int *mid_orig;           // midpoint -> reference node index
    const double *mid_drag;
    const double *node_ctf, *mid_ctf;      // 3 per vertex / midpoint: constant linear forces (or null)
    const int *vface_ptr, *vface;          // surface faces holding each vertex, in face order (or null)
    const int *mface_ptr, *mface;          // the same for midpoints
    const double *ff;                      // 3 per face: this step's constant surface force at each corner
    const int *lin_ptr;            // per vertex: its linearise events, in element order (or null)
    const int4 *lin_ev;            // up to three live midpoints (-1: already moved) summed into the vertex
    const void *mid_f;             // this step's midpoint forces (3 per midpoint, in the step's precision R) as
                                   // midpoint_force gives them, computed once by mid_force_kernel (or null)
    // a batch: reference node i belongs to the blob b with orig_off[b] <= i < orig_off[b + 1] (nblobs + 1
    // entries), draws from rng_state[6 b ..] and its chunk jumps start at chunk_jump[chunk_off[b]] (null: one blob)
    const int *orig_off;
    const int *chunk_off;
    int nblobs;
};

// force[i] -= RAND(-.5,.5) * sqrt(24 kT drag / dt), three components, for reference node i
// (Blob::aggregate_forces_and_solve, src/Blob.cpp:3190-3219); in a batch, i is the node's index in the
// concatenated numbering and the draws come from its blob's stream
template <class R>
__device__ __forceinline__ void stokes_noise_sub(const NodeForces &sn, int i, double drag, R (&F)[3]) {
    uint32_t base[6], s6[6];
    const uint32_t *rs = sn.rng_state;
    int li = i, chunk = i >> 5;
    if (sn.orig_off) {  // a batch: the node's blob, its index in the blob's numbering, the blob's stream
        int lo = 0, hi = sn.nblobs;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sn.orig_off[mid] <= i) lo = mid; else hi = mid;
        }
        li = i - sn.orig_off[lo];
        chunk = sn.chunk_off[lo] + (li >> 5);
        rs += 6 * (size_t)lo;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) s6[k] = rs[k];
    mrg_apply(sn.chunk_jump[chunk], s6, base);
    mrg_apply(sn.lane_jump[li & 31], base, s6);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double r = mrg_rand_half(s6);
        F[c] -= (R)(r * sqrt((24 * sn.kT * drag) / (sn.dt)));
    }
}

// force[node] += face force of every surface face holding the node, in face order
template <class R>
__device__ __forceinline__ void surface_add(const NodeForces &sn, const int *ptr, const int *faces, int i,
                                            R (&F)[3]) {
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const double *f = sn.ff + 3 * (size_t)faces[k];
#pragma unroll
        for (int c = 0; c < 3; ++c) F[c] += (R)f[c];
    }
}

// the force a midpoint carries into linearise_force: its constant forces, then its noise
template <class R>
__device__ __forceinline__ void midpoint_force(const NodeForces &sn, int m, R (&f)[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] = sn.mid_ctf ? (R)sn.mid_ctf[3 * (size_t)m + c] : (R)0;
    if (sn.mface_ptr) surface_add<R>(sn, sn.mface_ptr, sn.mface, m, f);
    if (sn.noise) stokes_noise_sub<R>(sn, sn.mid_orig[m], sn.mid_drag[m], f);
}

// the vertex's share of Blob::linearise_force (src/Blob.cpp:781-799): for each element holding the vertex,
// in element order, force += 0.5 * (f_m1 + f_m2 + f_m3) over that element's three midpoints at the vertex
// that still carry force (a midpoint's force is moved by the first element holding it, then zeroed)
template <class R>
__device__ __forceinline__ void midpoint_linearise(const NodeForces &sn, int a, R (&F)[3]) {
    for (int k = sn.lin_ptr[a]; k < sn.lin_ptr[a + 1]; ++k) {
        const int4 ev = sn.lin_ev[k];
        const int m[3] = {ev.x, ev.y, ev.z};
        R fm[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            fm[j][0] = fm[j][1] = fm[j][2] = (R)0;
            if (m[j] < 0) continue;
            if (sn.mid_f) {
                const R *mf = static_cast<const R *>(sn.mid_f) + 3 * (size_t)m[j];
                fm[j][0] = mf[0]; fm[j][1] = mf[1]; fm[j][2] = mf[2];
            } else {
                midpoint_force<R>(sn, m[j], fm[j]);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) F[c] += (R)0.5 * (fm[0][c] + fm[1][c] + fm[2][c]);
    }
}

// one rotational constant force on a node (CTF 2 of Blob::apply_ctforces, src/Blob.cpp:1684-1720)
struct RotEntry {
    double F;         // meso force
    double p[3];      // a point of the axis (meso length)
    double d[3];      // the axis' unit direction
    int torque;       // 0: F (r x d); 1: F / |r| (r x d)
    int pad;
};

// nodes (vertex rows, then midpoints) carrying rotational constant forces: each step their constant force is
// the linear sum plus every rotational force in file order, evaluated at the node's current position
struct RotArgs {
    int nv, nm;
    const int *v_row, *v_ptr;   // vertex row of list entry i, its forces [v_ptr[i], v_ptr[i + 1]) in ent
    const int *m_idx, *m_ptr;   // the same for midpoints (index into the midpoint list), ptr into ent_m
    const RotEntry *ent, *ent_m;
    const int *mid_a, *mid_b;   // midpoint edge ends (vertex rows)
    const double *px, *py, *pz;
    const double *lin_v, *lin_m;  // the static linear sums (3 per vertex / midpoint)
    double *out_v, *out_m;        // the step's constant forces (3 per vertex / midpoint)
    const DevStatus *st;
};

__device__ __forceinline__ void cross3(const double (&u)[3], const double (&v)[3], double (&w)[3]) {
    // arr3arr3VectorProduct, include/mat_vec_fns_II.h:369-373
    w[0] = u[1] * v[2] - v[1] * u[2];
    w[1] = -u[0] * v[2] + v[0] * u[2];
    w[2] = u[0] * v[1] - v[0] * u[1];
}

// magnitude (include/mat_vec_fns_II.h:326-333): an `omp simd` sum that GCC builds as (a0^2 + a2^2) + a1^2
__device__ __forceinline__ double magnitude3(const double (&a)[3]) { return sqrt((a[0] * a[0] + a[2] * a[2]) + a[1] * a[1]); }

// the force of one rotational entry on a node at p0: r to the nearest point of the axis
// (intersectingPointToLine, include/mat_vec_fns_II.h:755-777), then F (r x d) or F/|r| (r x d)
__device__ __forceinline__ void rot_force(const RotEntry &e, const double (&p0)[3], double (&f)[3]) {
    const double d[3] = {e.d[0], e.d[1], e.d[2]};
    double p0p1[3], v2[3], p3[3];
    for (int c = 0; c < 3; ++c) p0p1[c] = p0[c] - e.p[c];
    cross3(p0p1, d, v2);
    if (magnitude3(v2) < 3.0 * 2.220446049250313080847e-16) {  // ffea_const::threeErr
        for (int c = 0; c < 3; ++c) p3[c] = p0[c];
    } else {
        double cp3p0[3], v1v2[3];
        cross3(d, v2, cp3p0);
        cross3(d, cp3p0, v1v2);
        // detByRows (include/mat_vec_fns_II.h:379-385)
        double cc = p0p1[0] * (d[1] * v1v2[2] - d[2] * v1v2[1]);
        cc += p0p1[1] * (d[2] * v1v2[0] - d[0] * v1v2[2]);
        cc += p0p1[2] * (d[0] * v1v2[1] - d[1] * v1v2[0]);
        cc /= (v1v2[0] * v1v2[0] + v1v2[1] * v1v2[1] + v1v2[2] * v1v2[2]);
        for (int c = 0; c < 3; ++c) p3[c] = p0[c] + cc * cp3p0[c];
    }
    double r[3];
    for (int c = 0; c < 3; ++c) r[c] = p3[c] - p0[c];
    cross3(r, d, f);
    const double s = e.torque ? e.F / magnitude3(r) : e.F;
    for (int c = 0; c < 3; ++c) f[c] = s * f[c];
}

__global__ void __launch_bounds__(128) rot_force_kernel(RotArgs g);

// every midpoint's force of the step (midpoint_force) once, for the vertices' linearise replay to read
template <class R>
__global__ void __launch_bounds__(256) mid_force_kernel(NodeForces sn, int M, R *out, const DevStatus *st) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M || st->abort) return;
    R f[3];
    midpoint_force<R>(sn, m, f);
    out[3 * (size_t)m] = f[0];
    out[3 * (size_t)m + 1] = f[1];
    out[3 * (size_t)m + 2] = f[2];
}

// one step's constant surface forces (CTF 3 of Blob::apply_ctforces): each set's force spread over its faces in
// proportion to their current areas, area_j / (3 sum_k area_k) of it at each corner of face j
struct SurfArgs {
    int nsets, nfaces;
    const int *set_ptr, *set_faces;
    const double *set_force;       // 3 per set
    const int2 *corner;            // 3 per face: vertex rows (a, b) of the corner at (x_a + x_b) / 2
    const int *face_set_ptr, *face_set;
    const double *px, *py, *pz;
    double *set_total;             // per set
    double *ff;                    // 3 per face
    const DevStatus *st;
};

// Face::get_area (src/Face.cpp:169-187) at the current positions
__device__ __forceinline__ double face_area(const SurfArgs &g, int f) {
    double p[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int2 c = g.corner[3 * f + k];
        p[k][0] = .5 * (g.px[c.x] + g.px[c.y]);
        p[k][1] = .5 * (g.py[c.x] + g.py[c.y]);
        p[k][2] = .5 * (g.pz[c.x] + g.pz[c.y]);
    }
    double a[3], b[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        a[i] = p[1][i] - p[0][i];
        b[i] = p[2][i] - p[0][i];
    }
    const double t0 = a[1] * b[2] - a[2] * b[1], t1 = a[2] * b[0] - a[0] * b[2], t2 = a[0] * b[1] - a[1] * b[0];
    // magnitude (include/mat_vec_fns_II.h:326-333) is an `omp simd` reduction: built with GCC it sums two
    // lanes, (t0^2 + t2^2) + t1^2
    const double r = (t0 * t0 + t2 * t2) + t1 * t1;
    return .5 * sqrt(r);
}

__global__ void __launch_bounds__(128) surf_set_kernel(SurfArgs g);
__global__ void __launch_bounds__(128) surf_face_kernel(SurfArgs g);

template <class R>
struct GatherArgs {
    int N;
    int mode;             // 0: CG (NoMass or consistent mass), 1: mass-lumped scaling, 2: batch CG (f, r only)
    const int *inc_ptr, *inc;  // element*4 + slot, element order
    const R *ef;
    // mixed path: the element forces as per-block vertex sums, node-major (parts[part_ptr[a] ..
    // part_ptr[a + 1]) in block order), in place of inc / ef when set
    const float4 *parts;
    const int *part_ptr;
    const int *pinned;
    const double *drag;   // inertial Stokes drag (force -= v * drag) or null
    const double *vx, *vy, *vz;
    const R *dinv;        // Jacobi preconditioner (CG) or inverse lumped mass (mode 1)
    double *f;            // 4*N assembled force (solver input; the mixed gather: FP64 copy, or null)
    float *f32;           // mixed gather: the assembled force in FP32 in place of f (4*N), or null
    R *x, *r;
    double *partials;     // [0]: f.f, [stride]: r.z per block (mixed path: moments, float2 pairs)
    int stride;
    DevStatus *st;
    GridBarrier *gb;      // reset here for the CG launch that follows on the stream
    // mixed path only: node offsets from the reference point, positions, diagonal of V
    float4 *dpos;
    const double *px, *py, *pz;
    double xc[3];
    const R *diag;
    // Stokes noise (calc_stokes and calc_noise): 3 draws per node of the reference numbering, after the
    // elements' 7T, in node order; a midpoint's force is moved to its edge ends by linearise events
    NodeForces sn;
    // mixed mass-lumped step: the Euler update (euler_kernel's arithmetic) done by the gather, on these
    double *upx, *upy, *upz, *uvx, *uvy, *uvz;
    double dt;
    int fuse_euler;
    int threads;          // threads per block in mode 2 (0: the default); 64, 128 or 256
    // with fuse_euler: the next step's FP32 displacements from the rest positions nxr (3 x N, SoA) and velocities
    // (node_prep_kernel's arithmetic), or null
    float4 *nu, *nvf;
    const double *nxr;
    // with fuse_euler and noise: the next step's stream state at each 32-element chunk, ncj[c] (the chunk's jump
    // composed with the step's) applied to the step's state nrng (node_prep_kernel's other output), or null
    const MrgJump *ncj;
    const uint32_t *nrng;
    uint32_t *nchunk_state;
    int nnchunks;
    // with fuse_euler: the step closed here (finish_step_kernel's work) unless aborted: fin_jump applied to the step's
    // stream state nrng into fin_next (the other of two buffers, so no thread reads what is written) and the step
    // counted; or null
    const MrgJump *fin_jump;
    uint32_t *fin_next;
};

template <class R>
__global__ void __launch_bounds__(256) gather_kernel(GatherArgs<R> g) {
    __shared__ double smem[64];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a == 0 && g.gb) g.gb->count = 0u;
    double acc[2] = {0.0, 0.0};
    const bool live = a < g.N && !g.st->abort;
    if (live) {
        R F0 = 0, F1 = 0, F2 = 0;
        if (g.sn.node_ctf) {  // constant linear forces come first (apply_ctforces runs before the elements)
            F0 = (R)g.sn.node_ctf[3 * (size_t)a];
            F1 = (R)g.sn.node_ctf[3 * (size_t)a + 1];
            F2 = (R)g.sn.node_ctf[3 * (size_t)a + 2];
        }
        for (int m = g.inc_ptr[a]; m < g.inc_ptr[a + 1]; ++m) {
            const int es = g.inc[m];
            const R *c = g.ef + 12 * (size_t)(es >> 2) + 3 * (es & 3);
            F0 += c[0];
            F1 += c[1];
            F2 += c[2];
        }
        if (g.sn.vface_ptr) {
            R F[3] = {F0, F1, F2};
            surface_add<R>(g.sn, g.sn.vface_ptr, g.sn.vface, a, F);
            F0 = F[0]; F1 = F[1]; F2 = F[2];
        }
        if (g.drag) {  // inertial Stokes drag (src/Blob.cpp:3186-3188)
            const double dr = g.drag[a];
            F0 -= (R)(g.vx[a] * dr);
            F1 -= (R)(g.vy[a] * dr);
            F2 -= (R)(g.vz[a] * dr);
        }
        if (g.sn.on) {
            R F[3] = {F0, F1, F2};
            if (g.sn.noise) stokes_noise_sub<R>(g.sn, g.sn.node_orig[a], g.sn.node_drag[a], F);
            if (g.sn.lin_ptr) midpoint_linearise<R>(g.sn, a, F);
            F0 = F[0]; F1 = F[1]; F2 = F[2];
        }
        if (g.pinned[a]) { F0 = 0; F1 = 0; F2 = 0; }
        g.f[4 * a] = (double)F0;
        g.f[4 * a + 1] = (double)F1;
        g.f[4 * a + 2] = (double)F2;
        if (g.mode == 1) {  // MassLumpedSolver::solve, src/MassLumpedSolver.cpp:65-72
            g.x[4 * a] = F0 * g.dinv[4 * a];
            g.x[4 * a + 1] = F1 * g.dinv[4 * a + 1];
            g.x[4 * a + 2] = F2 * g.dinv[4 * a + 2];
        } else {  // conjugate_gradient_residual_assume_x_zero (src/NoMassCGSolver.cpp:196-220)
            const R z0 = g.dinv[4 * a] * F0, z1 = g.dinv[4 * a + 1] * F1, z2 = g.dinv[4 * a + 2] * F2;
            g.r[4 * a] = F0; g.r[4 * a + 1] = F1; g.r[4 * a + 2] = F2;
            g.x[4 * a] = 0; g.x[4 * a + 1] = 0; g.x[4 * a + 2] = 0;
            acc[0] = (double)(F0 * F0 + F1 * F1 + F2 * F2);
            acc[1] = (double)(F0 * z0 + F1 * z1 + F2 * z2);
        }
    }
    if (g.mode == 1) return;
    block_sum<2>(acc, smem);
    if (threadIdx.x == 0) {
        g.partials[blockIdx.x] = acc[0];
        g.partials[g.stride + blockIdx.x] = acc[1];
    }
}

// ---------------------------------------------------------------------------
// persistent Jacobi-PCG (NoMassCGSolver::solve :156-188 / ConjugateGradientSolver::solve :193-217)
//
// One cooperative launch runs the whole solve with two grid barriers per
// iteration: the search direction p = beta p + z of the previous iteration is
// not stored in a separate phase but recomputed on the fly, element by
// element, wherever the SpMV reads it (p lives in two buffers, old and new,
// which swap every iteration).
// ---------------------------------------------------------------------------
template <class R>
struct CgArgs {
    int N;
    int block3;           // 1: 3x3-block viscosity matrix, 0: scalar mass matrix applied per component
    int check_last;       // 1: also test convergence after the last allowed iteration (NoMass order)
    const int *slice_ptr, *rowlen, *bcol;
    const R *val;
    const R *dinv;        // Jacobi preconditioner, 4 per node
    const R *diag;        // mixed path: diagonal of V, 4 per node
    R *x, *r, *q;
    R *pbuf0, *pbuf1;     // search direction (mixed path: double-buffered; FP64 path: pbuf0 only)
    int tpn;              // threads per matrix row in the SpMV (1, 2, 4 or 8)
    const double *init_partials;  // from the gather kernel
    int n_init, init_stride;
    double *partials;     // per-block partial sums (float2 pairs on the mixed path)
    int stride;
    GridBarrier *gb;
    DevStatus *st;
    int imax;
    double eps2;
    unsigned long long limit_ns;
    double *history;      // |r|^2/|f|^2 per iteration (block 0 writes), capacity hist_cap
    int hist_cap;
    unsigned long long *phase_ns;  // FFEA_GPU_CG_PHASES timers of block 0 (thread 0), summed over iterations
    // mixed path: node offsets from the reference point and the rigid-mode coefficients (t, omega)
    const float4 *dpos;
    int nmodes;
    double modes[36];
    int npb;              // owned-rows kernels: rows owned by each block (a multiple of 32 / tpn)
    int sr;               // mixed path, 3x3-block matrix: the single-reduction kernel (cg_mixed_sr_kernel)
    // cg_mixed_sr_kernel: blocks owning a column of block b's rows (nb_ptr[b] .. nb_ptr[b + 1] in nb_list) and
    // one publication counter per block (FLAG_STRIDE words apart, zero at launch)
    const int *nb_ptr, *nb_list;
    unsigned int *flags;
    // cg_mixed_sr_kernel: degree of the Chebyshev polynomial preconditioner (0: Jacobi alone), its state
    // (CHEB_STATE doubles, zero at first) and the cost of one Chebyshev step relative to a Jacobi iteration
    int poly;
    double *cheb;
    float cheb_cost;
    int kc;               // cg_mixed_sr_kernel: 3x3 blocks per owned row kept in shared memory (0: none)
};

// p at node b for this iteration: p_new = beta p_old + D^{-1} r (vec3_scale_and_add with the
// preconditioned residual, src/NoMassCGSolver.cpp:181-183), or z itself on the first iteration.
template <class A, class R>
__device__ __forceinline__ void p_on_the_fly(const A &g, const R *pold, R beta, bool first, int b, R &p0, R &p1,
                                              R &p2) {
    const R z0 = g.dinv[4 * b] * g.r[4 * b], z1 = g.dinv[4 * b + 1] * g.r[4 * b + 1],
            z2 = g.dinv[4 * b + 2] * g.r[4 * b + 2];
    if (first) {
        p0 = z0; p1 = z1; p2 = z2;
    } else {
        p0 = fma(beta, pold[4 * b], z0);
        p1 = fma(beta, pold[4 * b + 1], z1);
        p2 = fma(beta, pold[4 * b + 2], z2);
    }
}

// Row a of q = V p, summed by the tpn lanes of a node group over blocks k = sub, sub + tpn, ... and
// combined with shuffles; every lane of the group returns the row. All 32 lanes of the warp call it
// together (rows past the end pass valid = false). ONTHEFLY: p is formed from p_old, r and D^{-1}
// (mixed path); otherwise it is read from pold (FP64 path).
template <bool ONTHEFLY, class A, class R>
__device__ __forceinline__ void spmv_row(const A &g, const R *pold, R beta, bool first, int a, int sub, bool valid,
                                         R &q0, R &q1, R &q2) {
    q0 = 0.0; q1 = 0.0; q2 = 0.0;
    const int tpn = g.tpn;
    if (valid) {
        const int s = a >> 5, lane = a & 31;
        const int base = g.slice_ptr[s];
        const int len = g.rowlen[a];
        if (g.block3 && ONTHEFLY) {
            // one block per trip, the next block's column index prefetched so that its dependent
            // loads can issue as soon as the current trip's loads are out
            const R *v = g.val + 9 * (size_t)base + lane;
            int k = sub;
            int bn = (k < len) ? g.bcol[base + 32 * k + lane] : 0;
#pragma unroll 1
            for (; k < len; k += tpn) {
                const int b = bn;
                if (k + tpn < len) bn = g.bcol[base + 32 * (k + tpn) + lane];
                const R *vk = v + (size_t)32 * 9 * k;
                const R v0 = vk[0], v1 = vk[32], v2 = vk[64], v3 = vk[96], v4 = vk[128], v5 = vk[160], v6 = vk[192],
                        v7 = vk[224], v8 = vk[256];
                R p0, p1, p2;
                p_on_the_fly(g, pold, beta, first, b, p0, p1, p2);
                q0 = fma(v0, p0, q0); q0 = fma(v1, p1, q0); q0 = fma(v2, p2, q0);
                q1 = fma(v3, p0, q1); q1 = fma(v4, p1, q1); q1 = fma(v5, p2, q1);
                q2 = fma(v6, p0, q2); q2 = fma(v7, p1, q2); q2 = fma(v8, p2, q2);
            }
        } else if (g.block3) {
            const R *v = g.val + 9 * (size_t)base + lane;
#pragma unroll 1
            for (int k = sub; k < len; k += tpn) {
                const int b = g.bcol[base + 32 * k + lane];
                const R *vk = v + (size_t)32 * 9 * k;
                const R v0 = vk[0], v1 = vk[32], v2 = vk[64], v3 = vk[96], v4 = vk[128], v5 = vk[160], v6 = vk[192],
                        v7 = vk[224], v8 = vk[256];
                R p0, p1, p2;
                if (ONTHEFLY) {
                    p_on_the_fly(g, pold, beta, first, b, p0, p1, p2);
                } else {
                    p0 = pold[4 * b]; p1 = pold[4 * b + 1]; p2 = pold[4 * b + 2];
                }
                q0 = fma(v0, p0, q0); q0 = fma(v1, p1, q0); q0 = fma(v2, p2, q0);
                q1 = fma(v3, p0, q1); q1 = fma(v4, p1, q1); q1 = fma(v5, p2, q1);
                q2 = fma(v6, p0, q2); q2 = fma(v7, p1, q2); q2 = fma(v8, p2, q2);
            }
        } else {
            const R *v = g.val + base + lane;
            for (int k = sub; k < len; k += tpn) {
                const int b = g.bcol[base + 32 * k + lane];
                const R m = v[32 * k];
                R p0, p1, p2;
                if (ONTHEFLY) {
                    p_on_the_fly(g, pold, beta, first, b, p0, p1, p2);
                } else {
                    p0 = pold[4 * b]; p1 = pold[4 * b + 1]; p2 = pold[4 * b + 2];
                }
                q0 = fma(m, p0, q0);
                q1 = fma(m, p1, q1);
                q2 = fma(m, p2, q2);
            }
        }
    }
    for (int o = 1; o < tpn; o <<= 1) {
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
        q2 += __shfl_xor_sync(0xffffffffu, q2, o);
    }
}

// Row (node) loop shared by every phase of the CG kernels. The W warps of the grid take consecutive
// runs of rppw = min(32 / tpn, ceil(N / W)) rows per pass, so that all SMs get the same number of rows;
// the tpn lanes of a row group work on the SpMV row together and its first lane (sub == 0) owns the
// node in the vector phases. All 32 lanes of a warp run every pass (rows past the end: valid = false).
#define FFEA_ROW_LOOP(g, a, sub, valid)                                                         \
    const int sub = (threadIdx.x & 31) % (g).tpn;                                               \
    const int wtot_ = (gridDim.x * blockDim.x) >> 5;                                            \
    const int rppw_ = min(32 / (g).tpn, ((g).N + wtot_ - 1) / wtot_);                           \
    const int wglob_ = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;                            \
    const int lrow_ = (threadIdx.x & 31) / (g).tpn;                                             \
    for (int a0_ = wglob_ * rppw_, a = a0_ + lrow_; a0_ < (g).N;                               \
         a0_ += wtot_ * rppw_, a = a0_ + lrow_)                                                 \
        for (bool valid = lrow_ < rppw_ && a < (g).N, once_ = true; once_; once_ = false)

#define FFEA_SPMV_LOOP FFEA_ROW_LOOP

// Node loop of the vector phases: the N nodes are split into gridDim.x equal runs, one per block,
// one node per thread (every block gets the same share; a phase's writes are read by other
// threads only after the grid barrier that ends the phase).
#define FFEA_NODE_LOOP(g, a)                                                                    \
    for (int npb_ = ((g).N + gridDim.x - 1) / gridDim.x, a = blockIdx.x * npb_ + threadIdx.x,    \
             aend_ = min((g).N, (blockIdx.x + 1) * npb_);                                       \
         a < aend_; a += blockDim.x)

constexpr int CG_MAX_THREADS = 1024;

constexpr int CG_PHASES = 10;  // the phase timers' slots (FFEA_GPU_CG_PHASES of the C ABI)

// Phase timers of block 0, thread 0: the time since the previous mark is added to a shared-memory slot k during
// the solve (a read-modify-write of phase_ns in global memory at every mark would hold block 0 for an L2 round
// trip each time) and the slots are added to phase_ns when the solve ends.
#define FFEA_PHASES_BEGIN(t_prev)                                                  \
    __shared__ unsigned long long s_phase_[CG_PHASES];                    \
    unsigned long long t_prev = 0ull;                                              \
    if (blockIdx.x == 0 && threadIdx.x == 0) {                                     \
        for (int k_ = 0; k_ < CG_PHASES; ++k_) s_phase_[k_] = 0ull;       \
        t_prev = globaltimer_ns();                                                 \
    }
#define FFEA_MARK(g, t_prev, k)                                                   \
    do {                                                                          \
        if (blockIdx.x == 0 && threadIdx.x == 0) {                                \
            const unsigned long long t_now_ = globaltimer_ns();                   \
            s_phase_[k] += t_now_ - (t_prev);                                     \
            (t_prev) = t_now_;                                                    \
        }                                                                         \
    } while (0)
#define FFEA_PHASES_END(g)                                                        \
    do {                                                                          \
        if (blockIdx.x == 0 && threadIdx.x == 0)                                  \
            for (int k_ = 0; k_ < CG_PHASES; ++k_) (g).phase_ns[k_] += s_phase_[k_]; \
    } while (0)

// FP64 CG: three phases (SpMV, residual update, direction update) with a grid barrier after each;
// every multiply-add is fused (the cross-node sums are reordered anyway, so the CG agrees with the
// reference to rounding, not bitwise).
template <class R>
__global__ void __launch_bounds__(1024, 1) cg_kernel(const __grid_constant__ CgArgs<R> g) {
    __shared__ double smem[2 * CG_MAX_THREADS];
    __shared__ double s_sc[4];
    __shared__ R s_alpha, s_beta;
    __shared__ double s_delta;
    __shared__ int s_conv;
    DevStatus *st = g.st;
    if (st->abort) return;
    FFEA_PHASES_BEGIN(tm);
    R *p = g.pbuf0;
    // p = z = D^{-1} r  (conjugate_gradient_residual_assume_x_zero, src/NoMassCGSolver.cpp:196-220)
    FFEA_NODE_LOOP(g, a) {
#pragma unroll
        for (int c = 0; c < 3; ++c) p[4 * a + c] = g.dinv[4 * a + c] * g.r[4 * a + c];
    }
    grid_sum_d<2>(g.init_partials, g.init_stride, g.n_init, s_sc);
    const double f2 = s_sc[0];
    if (threadIdx.x == 0) { s_delta = s_sc[1]; s_conv = 0; }
    unsigned int bar_ep = 0;  // grid barriers passed
    bool ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep);
    FFEA_MARK(g, tm, 0);
    int it = 0;
    for (; ok && it < g.imax; ++it) {
        // q = V p ; pTq   (get_alpha_denominator :253-266)
        double acc1[1] = {0.0};
        {
            FFEA_SPMV_LOOP(g, a, sub, valid) {
                R q0, q1, q2;
                spmv_row<false>(g, p, (R)0, false, a, sub, valid, q0, q1, q2);
                if (valid && sub == 0) {
                    g.q[4 * a] = q0; g.q[4 * a + 1] = q1; g.q[4 * a + 2] = q2;
                    acc1[0] += (double)fma(p[4 * a + 2], q2, fma(p[4 * a + 1], q1, p[4 * a] * q0));
                }
            }
        }
        FFEA_MARK(g, tm, 1);
        double out1[1];
        block_sum_smem<1>(acc1, smem, out1);
        if (threadIdx.x == 0) g.partials[blockIdx.x] = out1[0];
        FFEA_MARK(g, tm, 2);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 3);
        grid_sum_d<1>(g.partials, 0, gridDim.x, s_sc);
        if (threadIdx.x == 0) s_alpha = (R)(s_delta / s_sc[0]);
        __syncthreads();
        FFEA_MARK(g, tm, 4);
        const R alpha = s_alpha, malpha = -s_alpha;
        // x += alpha p ; r += (-alpha) q ; |r|^2 ; r.z   (vec3_add_to_scaled, residual2, apply_preconditioner)
        double acc2[2] = {0.0, 0.0};
        FFEA_NODE_LOOP(g, a) {
#pragma unroll
            for (int c = 0; c < 3; ++c) g.x[4 * a + c] = fma(alpha, p[4 * a + c], g.x[4 * a + c]);
            R r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                r[c] = fma(malpha, g.q[4 * a + c], g.r[4 * a + c]);
                g.r[4 * a + c] = r[c];
                z[c] = g.dinv[4 * a + c] * r[c];
            }
            acc2[0] += (double)fma(r[2], r[2], fma(r[1], r[1], r[0] * r[0]));
            acc2[1] += (double)fma(r[2], z[2], fma(r[1], z[1], r[0] * z[0]));
        }
        FFEA_MARK(g, tm, 5);
        double out2[2];
        block_sum_smem<2>(acc2, smem, out2);
        if (threadIdx.x == 0) {
            g.partials[g.stride + blockIdx.x] = out2[0];
            g.partials[2 * g.stride + blockIdx.x] = out2[1];
        }
        FFEA_MARK(g, tm, 6);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 7);
        grid_sum_d<2>(g.partials + g.stride, g.stride, gridDim.x, s_sc);
        if (threadIdx.x == 0) {
            const double res2 = (f2 == 0.0) ? 0.0 : s_sc[0] / f2;
            if (blockIdx.x == 0 && it < g.hist_cap) g.history[it] = res2;
            s_conv = (g.check_last || it + 1 < g.imax) && res2 < g.eps2;
            const double delta_old = s_delta;
            s_delta = s_sc[1];
            s_beta = (R)(s_delta / delta_old);
        }
        __syncthreads();
        FFEA_MARK(g, tm, 8);
        if (s_conv) {
            ++it;
            break;
        }
        // p = beta p + z   (vec3_scale_and_add :202-212)
        const R beta = s_beta;
        FFEA_NODE_LOOP(g, a) {
#pragma unroll
            for (int c = 0; c < 3; ++c) p[4 * a + c] = fma(beta, p[4 * a + c], g.dinv[4 * a + c] * g.r[4 * a + c]);
        }
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 9);
    }
    FFEA_PHASES_END(g);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!ok) {
            st->abort = 1;
        } else if (!s_conv) {
            st->cg_fail = 1;
            st->abort = 1;
            st->last_iters = g.imax;
            st->total_iters += g.imax;
        } else {
            st->last_iters = it;
            st->total_iters += it;
        }
    }
}

constexpr int FLAG_STRIDE = 32;  // words between two blocks' publication counters (one 128-byte line each)

// Block `blockIdx.x` has written its rows' z for round `epoch`: publish that (one release store after the
// block barrier), then wait (bounded by %globaltimer, acquire loads) until every block owning a column of its
// rows has published the same round; the closing barrier orders the block's later reads after those writes.
// Returns false on a timeout (recorded in st) or when another block recorded one.
template <class R>
__device__ __forceinline__ bool neighbour_sync(const CgArgs<R> &g, unsigned int epoch, DevStatus *st) {
    __syncthreads();
    if (threadIdx.x == 0)
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(g.flags + (size_t)FLAG_STRIDE * blockIdx.x),
                     "r"(epoch)
                     : "memory");
    int bad = 0;
    const int j0 = g.nb_ptr[blockIdx.x], j1 = g.nb_ptr[blockIdx.x + 1];
    for (int j = j0 + (int)threadIdx.x; j < j1 && !bad; j += blockDim.x) {
        const unsigned int *f = g.flags + (size_t)FLAG_STRIDE * g.nb_list[j];
        const unsigned long long t0 = globaltimer_ns();
        unsigned int polls = 0;
        for (;;) {
            unsigned int v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
            if ((int)(v - epoch) >= 0) break;
            if ((++polls & 255u) == 0u) {
                if (globaltimer_ns() - t0 > g.limit_ns) {
                    atomicExch(&st->timeout, 1);
                    atomicExch(&st->abort, 1);
                    bad = 1;
                    break;
                }
                if (*((volatile int *)&st->timeout)) { bad = 1; break; }
            }
        }
    }
    return __syncthreads_or(bad) == 0;
}

// Row a of q = V p for cg_own_kernel (FP64): the direction at neighbour b read as two 16-byte loads; the
// products are fused in the same order as spmv_row.
template <class R>
__device__ __forceinline__ void spmv_row_pd(const CgArgs<R> &g, const double2 *p2, int a, int sub, bool valid, R &q0,
                                            R &q1, R &q2) {
    q0 = 0.0; q1 = 0.0; q2 = 0.0;
    const int tpn = g.tpn;
    if (valid) {
        const int s = a >> 5, lane = a & 31;
        const int base = __ldg(g.slice_ptr + s);
        const int len = __ldg(g.rowlen + a);
        if (g.block3) {
            const R *v = g.val + 9 * (size_t)base + lane;
            int k = sub;
            int bn = (k < len) ? __ldg(g.bcol + base + 32 * k + lane) : 0;
#pragma unroll 1
            for (; k < len; k += tpn) {
                const int b = bn;
                if (k + tpn < len) bn = __ldg(g.bcol + base + 32 * (k + tpn) + lane);
                const R *vk = v + (size_t)32 * 9 * k;
                const R v0 = __ldg(vk), v1 = __ldg(vk + 32), v2 = __ldg(vk + 64), v3 = __ldg(vk + 96),
                        v4 = __ldg(vk + 128), v5 = __ldg(vk + 160), v6 = __ldg(vk + 192), v7 = __ldg(vk + 224),
                        v8 = __ldg(vk + 256);
                const double2 pa = p2[2 * b], pb = p2[2 * b + 1];
                const R p0 = pa.x, p1 = pa.y, p2v = pb.x;
                q0 = fma(v0, p0, q0); q0 = fma(v1, p1, q0); q0 = fma(v2, p2v, q0);
                q1 = fma(v3, p0, q1); q1 = fma(v4, p1, q1); q1 = fma(v5, p2v, q1);
                q2 = fma(v6, p0, q2); q2 = fma(v7, p1, q2); q2 = fma(v8, p2v, q2);
            }
        } else {
            const R *v = g.val + base + lane;
            for (int k = sub; k < len; k += tpn) {
                const int b = __ldg(g.bcol + base + 32 * k + lane);
                const R m = __ldg(v + 32 * k);
                const double2 pa = p2[2 * b], pb = p2[2 * b + 1];
                q0 = fma(m, (R)pa.x, q0);
                q1 = fma(m, (R)pa.y, q1);
                q2 = fma(m, (R)pb.x, q2);
            }
        }
    }
    for (int o = 1; o < tpn; o <<= 1) {
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
        q2 += __shfl_xor_sync(0xffffffffu, q2, o);
    }
}

// Bytes of dynamic shared memory cg_own_kernel needs for npb owned rows: x, r, q, p (FP64).
__host__ __device__ constexpr size_t own_smem_bytes_d(int npb) { return (size_t)12 * npb * sizeof(double); }

// The FP64 CG of cg_kernel with each block owning a fixed run of npb rows: their x, r, q and p stay in
// shared memory for the whole solve and the block computes its own rows' SpMV, so the residual and
// direction updates touch global memory only to publish p for the other blocks' SpMV (in the pbuf0 buffer,
// 32 bytes per node). Every value is computed by the same expression as in cg_kernel; only the grouping of
// the cross-node sums changes.
template <class R>
__global__ void __launch_bounds__(1024, 1) cg_own_kernel(const __grid_constant__ CgArgs<R> g) {
    static_assert(sizeof(R) == sizeof(double), "the FP64 owned-rows CG");
    extern __shared__ double snd[];
    __shared__ double smem[2 * CG_MAX_THREADS];
    __shared__ double s_sc[4];
    __shared__ R s_alpha, s_beta;
    __shared__ double s_delta;
    __shared__ int s_conv;
    DevStatus *st = g.st;
    if (st->abort) return;
    FFEA_PHASES_BEGIN(tm);
    const int npb = g.npb, a0 = blockIdx.x * npb;
    const int nloc = max(0, min(npb, g.N - a0));
    double *sx = snd, *sr = snd + 3 * npb, *sq = snd + 6 * npb, *sp = snd + 9 * npb;
    double2 *p2 = reinterpret_cast<double2 *>(g.pbuf0);
    // p = z = D^{-1} r  (conjugate_gradient_residual_assume_x_zero, src/NoMassCGSolver.cpp:196-220)
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
        const int a = a0 + l;
        R z[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const R r = g.r[4 * a + c];
            sr[c * npb + l] = r;
            sx[c * npb + l] = 0.0;
            z[c] = __ldg(g.dinv + 4 * a + c) * r;
            sp[c * npb + l] = z[c];
        }
        p2[2 * a] = make_double2(z[0], z[1]);
        p2[2 * a + 1] = make_double2(z[2], 0.0);
    }
    grid_sum_d<2>(g.init_partials, g.init_stride, g.n_init, s_sc);
    const double f2 = s_sc[0];
    if (threadIdx.x == 0) { s_delta = s_sc[1]; s_conv = 0; }
    unsigned int bar_ep = 0, nb_ep = 0;  // grid barriers passed, neighbour publications made
    bool ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep);
    const int tpn = g.tpn, gpb = blockDim.x / tpn, grp = threadIdx.x / tpn, sub = threadIdx.x % tpn;
    const int npass = (nloc + gpb - 1) / gpb;
    FFEA_MARK(g, tm, 0);
    int it = 0;
    for (; ok && it < g.imax; ++it) {
        // q = V p ; pTq   (get_alpha_denominator :253-266)
        double acc1[1] = {0.0};
        for (int ps = 0; ps < npass; ++ps) {
            const int l = ps * gpb + grp;
            const bool valid = l < nloc;
            R q0, q1, q2;
            spmv_row_pd(g, p2, a0 + l, sub, valid, q0, q1, q2);
            if (!valid || sub != 0) continue;
            sq[l] = q0; sq[npb + l] = q1; sq[2 * npb + l] = q2;
            acc1[0] += (double)fma(sp[2 * npb + l], q2, fma(sp[npb + l], q1, sp[l] * q0));
        }
        FFEA_MARK(g, tm, 1);
        double out1[1];
        block_sum_smem<1>(acc1, smem, out1);
        if (threadIdx.x == 0) g.partials[blockIdx.x] = out1[0];
        FFEA_MARK(g, tm, 2);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 3);
        grid_sum_d<1>(g.partials, 0, gridDim.x, s_sc);
        if (threadIdx.x == 0) s_alpha = (R)(s_delta / s_sc[0]);
        __syncthreads();
        FFEA_MARK(g, tm, 4);
        const R alpha = s_alpha, malpha = -s_alpha;
        // x += alpha p ; r += (-alpha) q ; |r|^2 ; r.z   (vec3_add_to_scaled, residual2, apply_preconditioner)
        double acc2[2] = {0.0, 0.0};
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            const int a = a0 + l;
            R r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sx[c * npb + l] = fma(alpha, sp[c * npb + l], sx[c * npb + l]);
                r[c] = fma(malpha, sq[c * npb + l], sr[c * npb + l]);
                sr[c * npb + l] = r[c];
                z[c] = __ldg(g.dinv + 4 * a + c) * r[c];
            }
            acc2[0] += (double)fma(r[2], r[2], fma(r[1], r[1], r[0] * r[0]));
            acc2[1] += (double)fma(r[2], z[2], fma(r[1], z[1], r[0] * z[0]));
        }
        FFEA_MARK(g, tm, 5);
        double out2[2];
        block_sum_smem<2>(acc2, smem, out2);
        if (threadIdx.x == 0) {
            g.partials[g.stride + blockIdx.x] = out2[0];
            g.partials[2 * g.stride + blockIdx.x] = out2[1];
        }
        FFEA_MARK(g, tm, 6);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 7);
        grid_sum_d<2>(g.partials + g.stride, g.stride, gridDim.x, s_sc);
        if (threadIdx.x == 0) {
            const double res2 = (f2 == 0.0) ? 0.0 : s_sc[0] / f2;
            if (blockIdx.x == 0 && it < g.hist_cap) g.history[it] = res2;
            s_conv = (g.check_last || it + 1 < g.imax) && res2 < g.eps2;
            const double delta_old = s_delta;
            s_delta = s_sc[1];
            s_beta = (R)(s_delta / delta_old);
        }
        __syncthreads();
        FFEA_MARK(g, tm, 8);
        if (s_conv) {
            ++it;
            break;
        }
        // p = beta p + z   (vec3_scale_and_add :202-212), published for the next SpMV
        const R beta = s_beta;
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            const int a = a0 + l;
            R pv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pv[c] = fma(beta, sp[c * npb + l], __ldg(g.dinv + 4 * a + c) * sr[c * npb + l]);
                sp[c * npb + l] = pv[c];
            }
            p2[2 * a] = make_double2(pv[0], pv[1]);
            p2[2 * a + 1] = make_double2(pv[2], 0.0);
        }
        // the next SpMV reads p only at the rows of the blocks owning its rows' columns: with their lists
        // (g.flags), wait for those blocks' publication rather than for the whole grid. Every block has finished
        // this iteration's SpMV (it precedes the two barriers above) before any block overwrites its p.
        if (g.flags) {
            if (!(ok = neighbour_sync(g, ++nb_ep, st))) break;
        } else if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) {
            break;
        }
        FFEA_MARK(g, tm, 9);
    }
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
        const int a = a0 + l;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            g.x[4 * a + c] = sx[c * npb + l];
            g.r[4 * a + c] = sr[c * npb + l];
        }
    }
    FFEA_PHASES_END(g);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!ok) {
            st->abort = 1;
        } else if (!s_conv) {
            st->cg_fail = 1;
            st->abort = 1;
            st->last_iters = g.imax;
            st->total_iters += g.imax;
        } else {
            st->last_iters = it;
            st->total_iters += it;
        }
    }
}

// ---------------------------------------------------------------------------
// Euler update (Blob::euler_integrate :3249-3279), non-finite check, RNG advance
// ---------------------------------------------------------------------------
template <class R>
struct EulerArgs {
    int N, nomass;
    double dt;
    const R *x;
    double *px, *py, *pz, *vx, *vy, *vz;
    uint32_t *rng_state;     // advanced by step_jump once per step
    const MrgJump *step_jump;
    DevStatus *st;
};

template <class R>
__global__ void __launch_bounds__(256) euler_kernel(EulerArgs<R> g) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (g.st->abort || g.st->cg_fail) return;
    if (a < g.N) {
        const double x0 = (double)g.x[4 * a], x1 = (double)g.x[4 * a + 1], x2 = (double)g.x[4 * a + 2];
        if (!(isfinite(x0) && isfinite(x1) && isfinite(x2))) atomicExch(&g.st->nonfinite, 1);
        if (g.nomass) {
            g.vx[a] = x0; g.vy[a] = x1; g.vz[a] = x2;
            g.px[a] += x0 * g.dt; g.py[a] += x1 * g.dt; g.pz[a] += x2 * g.dt;
        } else {
            g.vx[a] += x0 * g.dt; g.vy[a] += x1 * g.dt; g.vz[a] += x2 * g.dt;
            g.px[a] += g.vx[a] * g.dt; g.py[a] += g.vy[a] * g.dt; g.pz[a] += g.vz[a] * g.dt;
        }
    }
}

// ---------------------------------------------------------------------------
// measurements (Blob::make_measurements, src/Blob.cpp:1066-1202): strain energy, kinetic energy
// (inertial solvers), centroid of all nodes and the RMSD from the reference positions, as per-block
// FP64 sums in a fixed order (measure_kernel) and one block that adds them up (measure_final_kernel)
// ---------------------------------------------------------------------------
constexpr int MEASURE_NV = 6;  // strain energy, kinetic energy, sum x, sum y, sum z, sum |x - x0|^2

template <class R>
struct MeasureArgs {
    int T, N, M;              // elements, vertices, midpoints
    int inertial;
    const int4 *tet;
    const double *px, *py, *pz, *vx, *vy, *vz;
    const R *jinv, *G, *E, *vol0, *rho;
    const double *p0;         // 3 x N, SoA: reference positions of the vertices
    const int *mid_a, *mid_b; // midpoint edge ends (vertex indices)
    const double *m0;         // 3 x M, SoA: reference positions of the midpoints
    double *partials;         // MEASURE_NV rows of gridDim.x
};

// Twice the elastic energy of element i (the reference's measurement, halved by the caller): with F = J^T J0^-1
// and the volume ratio t = vol / vol0, vol0 (G (|F|^2 - 3) + C/2 (t^2 - 1) - (C + 2G) ln t), C = E - 2G/3.
// J and det J as calculate_jacobian forms them from the element's vertex rows t.
template <class R>
__device__ __forceinline__ double element_strain_energy2(int4 t, const double *px, const double *py, const double *pz,
                                                         const R *jinv, size_t T, int i, double Gs, double Es,
                                                         double v0) {
    const int nd[4] = {t.x, t.y, t.z, t.w};
    double J[3][3];
    for (int r = 0; r < 3; ++r) {
        J[r][0] = px[nd[r + 1]] - px[nd[0]];
        J[r][1] = py[nd[r + 1]] - py[nd[0]];
        J[r][2] = pz[nd[r + 1]] - pz[nd[0]];
    }
    const double d1 = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    const double d2 = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    const double d3 = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    const double det = J[0][0] * d1 + J[1][0] * d2 + J[2][0] * d3;
    const double vol = (1.0 / 6.0) * fabs(det);
    double F[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            F[a][b] = 0;
            for (int k = 0; k < 3; ++k) F[a][b] += J[k][a] * (double)jinv[(size_t)(3 * b + k) * T + i];
        }
    const double C = Es - (2.0 / 3.0) * Gs;
    const double t1 = vol / v0;
    const double ff = F[0][0] * F[0][0] + F[1][1] * F[1][1] + F[2][2] * F[2][2] + F[0][1] * F[0][1] +
                      F[1][0] * F[1][0] + F[0][2] * F[0][2] + F[2][0] * F[2][0] + F[1][2] * F[1][2] +
                      F[2][1] * F[2][1];
    return v0 * (Gs * (ff - 3) + 0.5 * C * (t1 * t1 - 1) - (C + 2 * Gs) * log(t1));
}

template <class R>
__global__ void __launch_bounds__(256) measure_kernel(MeasureArgs<R> g) {
    __shared__ double smem[MEASURE_NV * 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[MEASURE_NV] = {0, 0, 0, 0, 0, 0};
    if (i < g.T) {
        const int4 t = g.tet[i];
        const int nd[4] = {t.x, t.y, t.z, t.w};
        const double Gs = g.G[i], Es = g.E[i], v0 = g.vol0[i];
        if (g.inertial) {
            double v[12], tmp[12] = {0};
            for (int a = 0; a < 4; ++a) {
                v[a] = g.vx[nd[a]]; v[4 + a] = g.vy[nd[a]]; v[8 + a] = g.vz[nd[a]];
            }
            for (int k = 0; k < 12; k += 4)
                for (int a = 0; a < 4; ++a)
                    for (int b = 0; b < 4; ++b) tmp[a + k] += (a == b ? .1 : .05) * v[b + k];
            const double m = v0 * (double)g.rho[i];
            double s = 0;
            for (int k = 0; k < 12; ++k) s += v[k] * (tmp[k] * m);
            acc[1] = s;
        }
        acc[0] = element_strain_energy2<R>(t, g.px, g.py, g.pz, g.jinv, g.T, i, Gs, Es, v0);
    }
    if (i < g.N) {
        const double x = g.px[i], y = g.py[i], z = g.pz[i];
        const double dx = x - g.p0[i], dy = y - g.p0[g.N + i], dz = z - g.p0[2 * (size_t)g.N + i];
        acc[2] += x; acc[3] += y; acc[4] += z;
        acc[5] += dx * dx + dy * dy + dz * dz;
    }
    if (i < g.M) {
        const int a = g.mid_a[i], b = g.mid_b[i];
        const double x = .5 * (g.px[a] + g.px[b]), y = .5 * (g.py[a] + g.py[b]), z = .5 * (g.pz[a] + g.pz[b]);
        const double dx = x - g.m0[i], dy = y - g.m0[g.M + i], dz = z - g.m0[2 * (size_t)g.M + i];
        acc[2] += x; acc[3] += y; acc[4] += z;
        acc[5] += dx * dx + dy * dy + dz * dz;
    }
    block_sum<MEASURE_NV>(acc, smem);
    if (threadIdx.x == 0)
        for (int k = 0; k < MEASURE_NV; ++k) g.partials[k * gridDim.x + blockIdx.x] = acc[k];
}

// one block: the totals of measure_kernel's partials, halved energies (the reference's 1/2)
template <class R>
__global__ void __launch_bounds__(256) measure_final_kernel(const double *partials, int nb, double *out) {
    __shared__ double s[MEASURE_NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = wid; k < MEASURE_NV; k += nw) {
        double t = 0.0;
        for (int b = lane; b < nb; b += 32) t += partials[k * nb + b];
        t = warp_sum(t);
        if (lane == 0) s[k] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        out[0] = 0.5 * s[0];
        out[1] = 0.5 * s[1];
        for (int k = 2; k < MEASURE_NV; ++k) out[k] = s[k];
    }
}

// closes a step: RNG advance and step counter (one thread), after euler_kernel
__global__ void finish_step_kernel(uint32_t *rng_state, const MrgJump *step_jump, DevStatus *st);

}  // namespace ffea
