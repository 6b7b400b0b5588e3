// kernels_mixed.cuh -- the mixed-precision force gather and CG solve.
//
// The viscosity matrix V of a blob without Stokes drag is singular: rigid
// translations and rotations that leave every pinned node at rest produce no
// viscous stress, so V z = 0 for them (the columns of Z). The reference's FP64
// CG converges before rounding excites these directions; with V in FP32 the
// rounding of every product (~1e-7) feeds them and the 1e-10 relative
// residual becomes unreachable. This solver runs CG on
//     V~ = V + D Z G^{-1} Z^T D,     G = Z^T D Z,  D = diag(V),
// with the right-hand side projected to f^ = f - D Z G^{-1} Z^T f. V~ is
// symmetric positive definite, D^{-1} V~ maps each rigid mode to itself, and
// its solution x satisfies Z^T D x = 0 and V x = f^: exactly the solution the
// reference's Jacobi-PCG builds from x = 0 (its iterates stay in D^{-1} times
// the range of V, i.e. D-orthogonal to Z). With V~ nonsingular the whole CG
// can run in FP32: matrix, SpMV, x, r, p, q.
//
// Reductions: each node's contribution is formed in FP32, summed over the
// block and the grid as double-float pairs (two FP32 values, ~48-bit
// significand) and finished in FP64; GB300 runs FP64 at 1/64 of the FP32
// rate, so no per-node work touches the FP64 pipe. The scalars alpha, beta
// and the mode coefficients are computed once per block in FP64.
//
// Z is expressed through per-node offsets d_a from a reference point: the
// k-th mode is t_k + w_k x d_a. Z^T v needs only S1 = sum v_a and
// S2 = sum d_a x v_a; D Z c at node a is D_a (tau + Omega x d_a).
#pragma once

#include "kernels.cuh"

namespace ffea {

constexpr int MIXED_GATHER_NP = 28;  // f.f, S1_f(3), S2_f(3), M = sum Phi^T D Phi (21)
constexpr int MIXED_A_NP = 7;        // p.q, S1(Dp)(3), S2(Dp)(3)
constexpr int MIXED_B_NP = 2;        // r.r, r.z
// partial rows: [0, A) phase A, [A, A+B) phase B, A+B the initial r.z
constexpr int MIXED_PARTIAL_ROWS = MIXED_A_NP + MIXED_B_NP + 1;

// the six basis columns phi_j of Phi_a = [I | (.) x d]: e_x, e_y, e_z, e_x x d, e_y x d, e_z x d
__device__ __forceinline__ void phi_cols(float dx, float dy, float dz, float (&phi)[6][3]) {
    phi[0][0] = 1; phi[0][1] = 0; phi[0][2] = 0;
    phi[1][0] = 0; phi[1][1] = 1; phi[1][2] = 0;
    phi[2][0] = 0; phi[2][1] = 0; phi[2][2] = 1;
    phi[3][0] = 0; phi[3][1] = -dz; phi[3][2] = dy;
    phi[4][0] = dz; phi[4][1] = 0; phi[4][2] = -dx;
    phi[5][0] = -dy; phi[5][1] = dx; phi[5][2] = 0;
}

// mixed-path gather: f (FP64 copy) and r = f (FP32); node offsets; moments for the rigid-mode set-up
template <class R>
__global__ void __launch_bounds__(256) gather_mixed_kernel(GatherArgs<R> g) {
    __shared__ float2 smem[MIXED_GATHER_NP * 32];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a == 0 && g.gb) { g.gb->count = 0u; g.gb->passed = 0u; }
    df32 acc[MIXED_GATHER_NP];
#pragma unroll
    for (int i = 0; i < MIXED_GATHER_NP; ++i) acc[i] = df32{0.f, 0.f};
    if (a < g.N && !g.st->abort) {
        float F0 = 0, F1 = 0, F2 = 0;
        if (g.sn.node_ctf) {
            F0 = (float)g.sn.node_ctf[3 * (size_t)a];
            F1 = (float)g.sn.node_ctf[3 * (size_t)a + 1];
            F2 = (float)g.sn.node_ctf[3 * (size_t)a + 2];
        }
        for (int m = g.inc_ptr[a]; m < g.inc_ptr[a + 1]; ++m) {
            const int es = g.inc[m];
            const R *c = g.ef + 12 * (size_t)(es >> 2) + 3 * (es & 3);
            F0 += c[0];
            F1 += c[1];
            F2 += c[2];
        }
        if (g.sn.vface_ptr) {
            float F[3] = {F0, F1, F2};
            surface_add<float>(g.sn, g.sn.vface_ptr, g.sn.vface, a, F);
            F0 = F[0]; F1 = F[1]; F2 = F[2];
        }
        if (g.drag) {
            const double dr = g.drag[a];
            F0 -= (float)(g.vx[a] * dr);
            F1 -= (float)(g.vy[a] * dr);
            F2 -= (float)(g.vz[a] * dr);
        }
        if (g.sn.on) {
            float F[3] = {F0, F1, F2};
            if (g.sn.noise) stokes_noise_sub<float>(g.sn, g.sn.node_orig[a], g.sn.node_drag[a], F);
            if (g.sn.lin_ptr) midpoint_linearise<float>(g.sn, a, F);
            F0 = F[0]; F1 = F[1]; F2 = F[2];
        }
        if (g.pinned[a]) { F0 = 0; F1 = 0; F2 = 0; }
        g.f[4 * a] = F0; g.f[4 * a + 1] = F1; g.f[4 * a + 2] = F2;
        if (g.mode == 1) {
            g.x[4 * a] = F0 * g.dinv[4 * a];
            g.x[4 * a + 1] = F1 * g.dinv[4 * a + 1];
            g.x[4 * a + 2] = F2 * g.dinv[4 * a + 2];
            return;
        }
        g.r[4 * a] = F0; g.r[4 * a + 1] = F1; g.r[4 * a + 2] = F2;
        if (g.mode == 2) return;  // batch: the per-blob CG set-up forms the moments
        const float dx = (float)(g.px[a] - g.xc[0]), dy = (float)(g.py[a] - g.xc[1]), dz = (float)(g.pz[a] - g.xc[2]);
        g.dpos[a] = make_float4(dx, dy, dz, 0.f);
        acc[0] = df32{F0 * F0 + F1 * F1 + F2 * F2, 0.f};
        acc[1].hi = F0; acc[2].hi = F1; acc[3].hi = F2;
        acc[4].hi = dy * F2 - dz * F1; acc[5].hi = dz * F0 - dx * F2; acc[6].hi = dx * F1 - dy * F0;
        if (g.diag) {
            float phi[6][3];
            phi_cols(dx, dy, dz, phi);
            const float D[3] = {(float)g.diag[4 * a], (float)g.diag[4 * a + 1], (float)g.diag[4 * a + 2]};
            int k = 7;
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = i; j < 6; ++j, ++k)
                    acc[k].hi = phi[i][0] * D[0] * phi[j][0] + phi[i][1] * D[1] * phi[j][1] + phi[i][2] * D[2] * phi[j][2];
        }
    }
    if (g.mode != 0) return;
    df32 out[MIXED_GATHER_NP];
    block_sum_df<MIXED_GATHER_NP>(acc, smem, out);
    if (threadIdx.x == 0) {
        float2 *pp = reinterpret_cast<float2 *>(g.partials);
#pragma unroll
        for (int i = 0; i < MIXED_GATHER_NP; ++i) pp[i * g.stride + blockIdx.x] = make_float2(out[i].hi, out[i].lo);
    }
}

// The whole block, once per solve: G = Z^T D Z from the moments M, G^{-1} by Gauss-Jordan on the augmented
// [G | I] in shared memory (one thread per entry, one pivot at a time), A6 = modes^T G^{-1} modes, and
// (tau, Omega) of D Z c0 with c0 = G^{-1} Z^T f. Every thread of the block must call it; the results are
// in shared memory after it returns.
template <class A>
__device__ __noinline__ void mixed_setup(const A &g, const double *s_sc, double *s_A6, float *s_tau, float *s_Om, float *s_beta,
                            int *s_conv) {
    __shared__ double sM[36], sAug[6][12], sF[6], sV[6], sC[6], sPiv;
    const int t = threadIdx.x, k = g.nmodes;
    if (t < 36) {
        const int i = t / 6, j = t % 6, lo = i < j ? i : j, hi = i < j ? j : i;
        // packed upper triangle: row lo starts at 7 + lo*6 - lo*(lo-1)/2
        sM[t] = s_sc[7 + lo * 6 - (lo * (lo - 1)) / 2 + (hi - lo)];
    }
    __syncthreads();
    if (t < 36) {
        const int i = t / 6, j = t % 6;
        double sum = 0.0;
        if (i < k && j < k)
            for (int p = 0; p < 6; ++p)
                for (int q = 0; q < 6; ++q) sum += g.modes[6 * i + p] * sM[6 * p + q] * g.modes[6 * j + q];
        sAug[i][j] = sum;
        sAug[i][6 + j] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int col = 0; col < k; ++col) {
        if (t == 0) sPiv = sAug[col][col];
        __syncthreads();
        if (t < 12) sAug[col][t] /= sPiv;
        __syncthreads();
        if (t < 6) sF[t] = sAug[t][col];
        __syncthreads();
        if (t < 72) {
            const int i = t / 12, j = t % 12;
            if (i != col && i < k) sAug[i][j] -= sF[i] * sAug[col][j];
        }
        __syncthreads();
    }
    if (t < 36) {
        const int p = t / 6, q = t % 6;
        double sum = 0.0;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) sum += g.modes[6 * i + p] * sAug[i][6 + j] * g.modes[6 * j + q];
        s_A6[t] = sum;
    }
    if (t < 6) {
        const double *m = g.modes + 6 * t;
        sV[t] = (t < k) ? m[0] * s_sc[1] + m[1] * s_sc[2] + m[2] * s_sc[3] + m[3] * s_sc[4] + m[4] * s_sc[5] +
                              m[5] * s_sc[6]
                        : 0.0;
    }
    __syncthreads();
    if (t < 6) {
        double c = 0.0;
        for (int j = 0; j < k; ++j) c += sAug[t][6 + j] * sV[j];
        sC[t] = (t < k) ? c : 0.0;
    }
    __syncthreads();
    if (t < 6) {
        double sum = 0.0;
        for (int i = 0; i < k; ++i) sum += sC[i] * g.modes[6 * i + t];
        if (t < 3) s_tau[t] = (float)sum; else s_Om[t - 3] = (float)sum;
    }
    if (t == 0) {
        *s_beta = 0.f;
        *s_conv = 0;
    }
    __syncthreads();
}

template <class R>
__global__ void __launch_bounds__(1024, 1) cg_mixed_kernel(const __grid_constant__ CgArgs<R> g) {
    __shared__ float smemf[MIXED_A_NP * 32];
    __shared__ double s_sc[MIXED_GATHER_NP];
    __shared__ double s_A6[36];
    __shared__ float s_alpha, s_beta, s_tau[3], s_Om[3];
    __shared__ double s_delta;
    __shared__ int s_conv;
    DevStatus *st = g.st;
    if (st->abort) return;
    const bool defl = g.nmodes > 0;
    unsigned long long tm = (blockIdx.x == 0 && threadIdx.x == 0) ? globaltimer_ns() : 0ull;
    float2 *partials = reinterpret_cast<float2 *>(g.partials);
    // set-up: G = Z^T D Z from the moments M, projected right-hand side
    grid_sum_df<MIXED_GATHER_NP>(reinterpret_cast<const float2 *>(g.init_partials), g.init_stride, g.n_init, s_sc);
    const double f2 = s_sc[0];
    mixed_setup(g, s_sc, s_A6, s_tau, s_Om, &s_beta, &s_conv);
    float acc0[1] = {0.f};
    FFEA_NODE_LOOP(g, a) {
        float r0 = g.r[4 * a], r1 = g.r[4 * a + 1], r2 = g.r[4 * a + 2];
        if (defl) {
            const float4 d = g.dpos[a];
            r0 -= g.diag[4 * a] * (s_tau[0] + (s_Om[1] * d.z - s_Om[2] * d.y));
            r1 -= g.diag[4 * a + 1] * (s_tau[1] + (s_Om[2] * d.x - s_Om[0] * d.z));
            r2 -= g.diag[4 * a + 2] * (s_tau[2] + (s_Om[0] * d.y - s_Om[1] * d.x));
            g.r[4 * a] = r0; g.r[4 * a + 1] = r1; g.r[4 * a + 2] = r2;
        }
        g.x[4 * a] = 0.f; g.x[4 * a + 1] = 0.f; g.x[4 * a + 2] = 0.f;
        acc0[0] += r0 * (g.dinv[4 * a] * r0) + r1 * (g.dinv[4 * a + 1] * r1) + r2 * (g.dinv[4 * a + 2] * r2);
    }
    const int row0 = MIXED_A_NP + MIXED_B_NP;
    {
        df32 o[1];
        block_reduce_f<1>(acc0, smemf, o);
        if (threadIdx.x == 0) partials[row0 * g.stride + blockIdx.x] = make_float2(o[0].hi, o[0].lo);
    }
    bool ok = grid_sync(g.gb, st, g.limit_ns);
    if (ok) {
        grid_sum_df<1>(partials + row0 * g.stride, 0, gridDim.x, s_sc);
        if (threadIdx.x == 0) s_delta = s_sc[0];
        __syncthreads();
    }
    float *pold = g.pbuf0, *pnew = g.pbuf1;
    FFEA_MARK(g, tm, 0);
    int it = 0;
    for (; ok && it < g.imax; ++it) {
        const bool first = it == 0;
        const float beta = s_beta;
        // phase A: q = V p with p formed on the fly; p.q; moments of D p for Z^T D p
        float acc[MIXED_A_NP];
#pragma unroll
        for (int i = 0; i < MIXED_A_NP; ++i) acc[i] = 0.f;
        {
            FFEA_SPMV_LOOP(g, a, sub, valid) {
                float q0, q1, q2;
                spmv_row<true>(g, pold, beta, first, a, sub, valid, q0, q1, q2);
                if (!valid || sub != 0) continue;
                float p0, p1, p2;
                p_on_the_fly(g, pold, beta, first, a, p0, p1, p2);
                pnew[4 * a] = p0; pnew[4 * a + 1] = p1; pnew[4 * a + 2] = p2;
                g.q[4 * a] = q0; g.q[4 * a + 1] = q1; g.q[4 * a + 2] = q2;
                acc[0] += p0 * q0 + p1 * q1 + p2 * q2;
                if (defl) {
                    const float4 d = g.dpos[a];
                    const float e0 = g.diag[4 * a] * p0, e1 = g.diag[4 * a + 1] * p1, e2 = g.diag[4 * a + 2] * p2;
                    acc[1] += e0; acc[2] += e1; acc[3] += e2;
                    acc[4] += d.y * e2 - d.z * e1;
                    acc[5] += d.z * e0 - d.x * e2;
                    acc[6] += d.x * e1 - d.y * e0;
                }
            }
        }
        FFEA_MARK(g, tm, 1);
        {
            df32 o[MIXED_A_NP];
            block_reduce_f<MIXED_A_NP>(acc, smemf, o);
            if (threadIdx.x == 0)
#pragma unroll
                for (int i = 0; i < MIXED_A_NP; ++i) partials[i * g.stride + blockIdx.x] = make_float2(o[i].hi, o[i].lo);
        }
        FFEA_MARK(g, tm, 2);
        if (!(ok = grid_sync(g.gb, st, g.limit_ns))) break;
        FFEA_MARK(g, tm, 3);
        grid_sum_df<MIXED_A_NP>(partials, g.stride, gridDim.x, s_sc);
        // (tau, Omega) = A6 S over six lanes of warp 0; p.V~p = p.q + S . (tau, Omega); alpha = delta / p.V~p
        if (threadIdx.x < 32) {
            const int l = threadIdx.x;
            double tO = 0.0;
            if (defl && l < 6) {
#pragma unroll
                for (int q = 0; q < 6; ++q) tO += s_A6[6 * l + q] * s_sc[1 + q];
            }
            double prod = (l < 6) ? tO * s_sc[1 + l] : 0.0;
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) prod += __shfl_xor_sync(0xffffffffu, prod, o);
            if (l < 6) {
                if (l < 3) s_tau[l] = (float)tO; else s_Om[l - 3] = (float)tO;
            }
            if (l == 0) s_alpha = (float)s_delta / (float)(s_sc[0] + prod);
        }
        __syncthreads();
        FFEA_MARK(g, tm, 4);
        const float alpha = s_alpha;
        const float t0 = s_tau[0], t1 = s_tau[1], t2 = s_tau[2], O0 = s_Om[0], O1 = s_Om[1], O2 = s_Om[2];
        // phase B: x += alpha p ; r -= alpha (q + D (tau + Omega x d)) ; r.r ; r.z
        float acc2[MIXED_B_NP] = {0.f, 0.f};
        FFEA_NODE_LOOP(g, a) {
#pragma unroll
            for (int c = 0; c < 3; ++c) g.x[4 * a + c] += alpha * pnew[4 * a + c];
            float q0 = g.q[4 * a], q1 = g.q[4 * a + 1], q2 = g.q[4 * a + 2];
            if (defl) {
                const float4 d = g.dpos[a];
                q0 += g.diag[4 * a] * (t0 + (O1 * d.z - O2 * d.y));
                q1 += g.diag[4 * a + 1] * (t1 + (O2 * d.x - O0 * d.z));
                q2 += g.diag[4 * a + 2] * (t2 + (O0 * d.y - O1 * d.x));
            }
            const float r0 = g.r[4 * a] - alpha * q0, r1 = g.r[4 * a + 1] - alpha * q1, r2 = g.r[4 * a + 2] - alpha * q2;
            g.r[4 * a] = r0; g.r[4 * a + 1] = r1; g.r[4 * a + 2] = r2;
            acc2[0] += r0 * r0 + r1 * r1 + r2 * r2;
            acc2[1] += r0 * (g.dinv[4 * a] * r0) + r1 * (g.dinv[4 * a + 1] * r1) + r2 * (g.dinv[4 * a + 2] * r2);
        }
        FFEA_MARK(g, tm, 5);
        {
            df32 o[MIXED_B_NP];
            block_reduce_f<MIXED_B_NP>(acc2, smemf, o);
            if (threadIdx.x == 0)
                for (int i = 0; i < MIXED_B_NP; ++i)
                    partials[(MIXED_A_NP + i) * g.stride + blockIdx.x] = make_float2(o[i].hi, o[i].lo);
        }
        FFEA_MARK(g, tm, 6);
        if (!(ok = grid_sync(g.gb, st, g.limit_ns))) break;
        FFEA_MARK(g, tm, 7);
        grid_sum_df<MIXED_B_NP>(partials + MIXED_A_NP * g.stride, g.stride, gridDim.x, s_sc);
        if (threadIdx.x == 0) {
            // |r|^2/|f|^2 < epsilon2 tested as |r|^2 < epsilon2 |f|^2 (f2 == 0 counts as converged)
            s_conv = (g.check_last || it + 1 < g.imax) && (f2 == 0.0 || s_sc[0] < g.eps2 * f2);
            if (blockIdx.x == 0 && it < g.hist_cap) g.history[it] = (f2 == 0.0) ? 0.0 : s_sc[0] / f2;
            const double delta_old = s_delta;
            s_delta = s_sc[1];
            s_beta = (float)s_delta / (float)delta_old;
        }
        __syncthreads();
        FFEA_MARK(g, tm, 8);
        if (s_conv) {
            ++it;
            break;
        }
        float *t = pold; pold = pnew; pnew = t;
    }
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

}  // namespace ffea
