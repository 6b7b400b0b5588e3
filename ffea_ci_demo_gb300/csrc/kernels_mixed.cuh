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
#include "kernels_element_mixed.cuh"

namespace ffea {

constexpr int MIXED_GATHER_NP = 28;  // f.f, S1_f(3), S2_f(3), M = sum Phi^T D Phi (21)
constexpr int MIXED_A_NP = 7;        // p.q, S1(Dp)(3), S2(Dp)(3)
constexpr int MIXED_B_NP = 2;        // r.r, r.z
// partial rows: [0, A) phase A, [A, A+B) phase B, A+B the initial r.z
constexpr int MIXED_PARTIAL_ROWS = MIXED_A_NP + MIXED_B_NP + 1;
// cg_mixed_sr_kernel's one reduction per iteration: r.z, r.r, z.w, z.q, p.w, S1(Dz)(3), S2(Dz)(3)
constexpr int MIXED_SR_NP = 11;

// the six basis columns phi_j of Phi_a = [I | (.) x d]: e_x, e_y, e_z, e_x x d, e_y x d, e_z x d
__device__ __forceinline__ void phi_cols(float dx, float dy, float dz, float (&phi)[6][3]) {
    phi[0][0] = 1; phi[0][1] = 0; phi[0][2] = 0;
    phi[1][0] = 0; phi[1][1] = 1; phi[1][2] = 0;
    phi[2][0] = 0; phi[2][1] = 0; phi[2][2] = 1;
    phi[3][0] = 0; phi[3][1] = -dz; phi[3][2] = dy;
    phi[4][0] = dz; phi[4][1] = 0; phi[4][2] = -dx;
    phi[5][0] = -dy; phi[5][1] = dx; phi[5][2] = 0;
}

// mixed-path gather: f (FP64 copy) and r = f (FP32); node offsets; moments for the rigid-mode set-up. MODE is
// g.mode: 0 (one blob's CG, with the block moments), 1 (mass-lumped), 2 (batch CG); the modes without the block
// reduction carry none of its registers. NF: some node force besides the elements' (constant forces, inertial
// Stokes drag, Stokes noise, midpoint forces); without, none of their registers either, and the mass-lumped form
// is held to 32 registers (a full SM of threads; 1 % faster than 40 registers on the 64^3 step).
template <class R, int MODE, bool NF>
__global__ void __launch_bounds__(256, (MODE == 1 && !NF) ? 8 : 1) gather_mixed_kernel(GatherArgs<R> g) {
    __shared__ float2 smem[MIXED_GATHER_NP * 32];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a == 0 && g.gb) g.gb->count = 0u;
    if constexpr (MODE == 1) {
        if (g.fin_next && a == 0 && !g.st->abort) {
            uint32_t s6[6], o6[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) s6[k] = g.nrng[k];
            mrg_apply(*g.fin_jump, s6, o6);
#pragma unroll
            for (int k = 0; k < 6; ++k) g.fin_next[k] = o6[k];
            g.st->steps_done += 1;
        }
        if (g.nchunk_state && a < g.nnchunks) {
            uint32_t s6[6], o6[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) s6[k] = g.nrng[k];
            mrg_apply(g.ncj[a], s6, o6);
#pragma unroll
            for (int k = 0; k < 6; ++k) g.nchunk_state[6 * (size_t)a + k] = o6[k];
        }
    }
    df32 acc[MIXED_GATHER_NP];
#pragma unroll
    for (int i = 0; i < MIXED_GATHER_NP; ++i) acc[i] = df32{0.f, 0.f};
    if (a < g.N && !g.st->abort) {
        float F0 = 0, F1 = 0, F2 = 0;
        if (NF && g.sn.node_ctf) {
            F0 = (float)g.sn.node_ctf[3 * (size_t)a];
            F1 = (float)g.sn.node_ctf[3 * (size_t)a + 1];
            F2 = (float)g.sn.node_ctf[3 * (size_t)a + 2];
        }
        if (g.parts) {
            // two block sums per trip, both loads ahead of the adds (the adds keep block order)
            int m = g.part_ptr[a];
            const int m1 = g.part_ptr[a + 1];
            for (; m + 2 <= m1; m += 2) {
                const float4 q = g.parts[m], q2 = g.parts[m + 1];
                F0 += q.x; F1 += q.y; F2 += q.z;
                F0 += q2.x; F1 += q2.y; F2 += q2.z;
            }
            if (m < m1) {
                const float4 q = g.parts[m];
                F0 += q.x; F1 += q.y; F2 += q.z;
            }
        } else {
            for (int m = g.inc_ptr[a]; m < g.inc_ptr[a + 1]; ++m) {
                const int es = g.inc[m];
                const R *c = g.ef + 12 * (size_t)(es >> 2) + 3 * (es & 3);
                F0 += c[0];
                F1 += c[1];
                F2 += c[2];
            }
        }
        if (NF && g.sn.vface_ptr) {
            float F[3] = {F0, F1, F2};
            surface_add<float>(g.sn, g.sn.vface_ptr, g.sn.vface, a, F);
            F0 = F[0]; F1 = F[1]; F2 = F[2];
        }
        if (NF && g.drag) {
            const double dr = g.drag[a];
            F0 -= (float)(g.vx[a] * dr);
            F1 -= (float)(g.vy[a] * dr);
            F2 -= (float)(g.vz[a] * dr);
        }
        if (NF && g.sn.on) {
            float F[3] = {F0, F1, F2};
            if (g.sn.noise) stokes_noise_sub<float>(g.sn, g.sn.node_orig[a], g.sn.node_drag[a], F);
            if (g.sn.lin_ptr) midpoint_linearise<float>(g.sn, a, F);
            F0 = F[0]; F1 = F[1]; F2 = F[2];
        }
        if (g.pinned[a]) { F0 = 0; F1 = 0; F2 = 0; }
        if (g.f32) {
            g.f32[4 * a] = F0; g.f32[4 * a + 1] = F1; g.f32[4 * a + 2] = F2;
        } else if (g.f) {
            g.f[4 * a] = F0; g.f[4 * a + 1] = F1; g.f[4 * a + 2] = F2;
        }
        if constexpr (MODE == 1) {
            const float4 di = reinterpret_cast<const float4 *>(g.dinv)[a];
            const R x0 = F0 * di.x, x1 = F1 * di.y, x2 = F2 * di.z;
            g.x[4 * a] = x0;
            g.x[4 * a + 1] = x1;
            g.x[4 * a + 2] = x2;
            if (g.fuse_euler) {
                // euler_integrate (src/Blob.cpp:3249-3279) as euler_kernel does it: v += a dt, p += v dt
                if (!(isfinite(x0) && isfinite(x1) && isfinite(x2))) atomicExch(&g.st->nonfinite, 1);
                const double a0 = (double)x0, a1 = (double)x1, a2 = (double)x2;
                const double v0 = g.uvx[a] + a0 * g.dt, v1 = g.uvy[a] + a1 * g.dt, v2 = g.uvz[a] + a2 * g.dt;
                g.uvx[a] = v0; g.uvy[a] = v1; g.uvz[a] = v2;
                const double p0 = g.upx[a] + v0 * g.dt, p1 = g.upy[a] + v1 * g.dt, p2 = g.upz[a] + v2 * g.dt;
                g.upx[a] = p0; g.upy[a] = p1; g.upz[a] = p2;
                if (g.nu) {
                    const size_t N = g.N;
                    g.nu[a] = make_float4((float)(p0 - g.nxr[a]), (float)(p1 - g.nxr[N + a]),
                                          (float)(p2 - g.nxr[2 * N + a]), 0.f);
                    g.nvf[a] = make_float4((float)v0, (float)v1, (float)v2, 0.f);
                }
            }
            return;
        }
        g.r[4 * a] = F0; g.r[4 * a + 1] = F1; g.r[4 * a + 2] = F2;
        if constexpr (MODE == 2) return;  // batch: the per-blob CG set-up forms the moments
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
    if constexpr (MODE != 0) return;
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
    FFEA_PHASES_BEGIN(tm);
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
    unsigned int bar_ep = 0;  // grid barriers passed
    bool ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep);
    if (ok) {
        grid_sum_df<1>(partials + row0 * g.stride, 0, gridDim.x, s_sc);
        if (threadIdx.x == 0) s_delta = s_sc[0];
        __syncthreads();
    }
    float *pold = g.pbuf0, *pnew = g.pbuf1;
    FFEA_MARK(g, tm, 0);
    int it = 0;
    // a zero force (a blob exactly at rest without noise) has the solution x = 0: no iteration (the first step
    // length would be 0/0)
    if (f2 == 0.0 && threadIdx.x == 0) s_conv = 1;
    for (; ok && it < g.imax && f2 != 0.0; ++it) {
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
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
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
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
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

// Block reduction of NV FP32 per-thread values straight into the per-block partial rows: FP32 within
// each warp, then warp w sums values w, w + (warps), ... over the warps in double-float and its lane 0
// stores the pairs. The caller must pass a __syncthreads() before smem is written again.
template <int NV>
__device__ __forceinline__ void block_reduce_store(const float (&v)[NV], float *smem, float2 *partials, int stride,
                                                   int row0) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const float w = warp_sum_f(v[i]);
        if (lane == 0) smem[i * 32 + wid] = w;
    }
    __syncthreads();
    for (int i = wid; i < NV; i += nw) {
        df32 t = {lane < nw ? smem[i * 32 + lane] : 0.f, 0.f};
        t = warp_sum_df(t);
        if (lane == 0) partials[(row0 + i) * stride + blockIdx.x] = make_float2(t.hi, t.lo);
    }
}

// grid_sum_df with each lane's loads issued eight at a time before their sums: the same fixed order, the
// partials' L2 latency paid once per 256 blocks.
template <int NV>
__device__ __forceinline__ void grid_sum_df8(const float2 *partials, int stride, int nb, double *s_out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wid; i < NV; i += nw) {
        df32 t = {0.f, 0.f};
        for (int b0 = 0; b0 < nb; b0 += 256) {
            float2 q[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int b = b0 + lane + 32 * j;
                q[j] = (b < nb) ? __ldcg(partials + i * stride + b) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) t = df_add(t, df32{q[j].x, q[j].y});
        }
        t = warp_sum_df(t);
        if (lane == 0) s_out[i] = (double)t.hi + (double)t.lo;
    }
    __syncthreads();
}

// The same row with U blocks per trip (3x3 blocks only): all U blocks' loads (columns, values, z and p) issue
// before any of their products, so U of the row's dependent DRAM round trips overlap; the products are
// accumulated in spmv_row_z's order, so the result is identical.
template <int U, class A>
__device__ __forceinline__ void spmv_row_zu(const A &g, const float4 *z4, const float4 *p4, float beta, bool first,
                                            int a, int sub, bool valid, float &q0, float &q1, float &q2) {
    q0 = 0.f; q1 = 0.f; q2 = 0.f;
    const int tpn = g.tpn;
    if (valid) {
        const int s = a >> 5, lane = a & 31;
        const int base = __ldg(g.slice_ptr + s);
        const int len = __ldg(g.rowlen + a);
        const float *v = g.val + 9 * (size_t)base + lane;
#pragma unroll 1
        for (int k = sub; k < len; k += U * tpn) {
            int bc[U];
            float w[U][9];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int ku = k + u * tpn;
                const bool in = ku < len;
                bc[u] = in ? __ldg(g.bcol + base + 32 * ku + lane) : 0;
                const float *vk = v + (size_t)32 * 9 * ku;
#pragma unroll
                for (int i = 0; i < 9; ++i) w[u][i] = in ? __ldg(vk + 32 * i) : 0.f;
            }
            float pz[U][3];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const float4 z = z4[bc[u]];
                pz[u][0] = z.x; pz[u][1] = z.y; pz[u][2] = z.z;
                if (!first) {
                    const float4 po = p4[bc[u]];
                    pz[u][0] = fmaf(beta, po.x, pz[u][0]);
                    pz[u][1] = fmaf(beta, po.y, pz[u][1]);
                    pz[u][2] = fmaf(beta, po.z, pz[u][2]);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (k + u * tpn >= len) break;
                q0 = fmaf(w[u][0], pz[u][0], q0); q0 = fmaf(w[u][1], pz[u][1], q0); q0 = fmaf(w[u][2], pz[u][2], q0);
                q1 = fmaf(w[u][3], pz[u][0], q1); q1 = fmaf(w[u][4], pz[u][1], q1); q1 = fmaf(w[u][5], pz[u][2], q1);
                q2 = fmaf(w[u][6], pz[u][0], q2); q2 = fmaf(w[u][7], pz[u][1], q2); q2 = fmaf(w[u][8], pz[u][2], q2);
            }
        }
    }
    for (int o = 1; o < tpn; o <<= 1) {
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
        q2 += __shfl_xor_sync(0xffffffffu, q2, o);
    }
}

// Row a of q = V p for cg_mixed_own_kernel and cg_batch_kernel: p at a neighbour b is formed from the preconditioned residual
// z_b and the previous direction, both stored as float4 per node (two 16-byte loads per neighbour).
// The same row with two blocks per trip: both blocks' loads (values, columns, z and p) issue before
// either block's products, halving the chain of dependent L2 round trips per lane. The products are
// accumulated in the same order as spmv_row_z, so the result is identical.
template <class A>
__device__ __forceinline__ void spmv_row_z2(const A &g, const float4 *z4, const float4 *p4, float beta, bool first,
                                            int a, int sub, bool valid, float &q0, float &q1, float &q2) {
    q0 = 0.f; q1 = 0.f; q2 = 0.f;
    const int tpn = g.tpn;
    if (valid) {
        const int s = a >> 5, lane = a & 31;
        const int base = __ldg(g.slice_ptr + s);
        const int len = __ldg(g.rowlen + a);
        const float *v = g.val + 9 * (size_t)base + lane;
        int k = sub;
#pragma unroll 1
        for (; k + tpn < len; k += 2 * tpn) {
            const int ba = __ldg(g.bcol + base + 32 * k + lane), bb = __ldg(g.bcol + base + 32 * (k + tpn) + lane);
            const float *va = v + (size_t)32 * 9 * k, *vb = v + (size_t)32 * 9 * (k + tpn);
            float wa[9], wb[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                wa[i] = __ldg(va + 32 * i);
                wb[i] = __ldg(vb + 32 * i);
            }
            const float4 za = z4[ba], zb = z4[bb];
            float pa0 = za.x, pa1 = za.y, pa2 = za.z, pb0 = zb.x, pb1 = zb.y, pb2 = zb.z;
            if (!first) {
                const float4 oa = p4[ba], ob = p4[bb];
                pa0 = fmaf(beta, oa.x, pa0); pa1 = fmaf(beta, oa.y, pa1); pa2 = fmaf(beta, oa.z, pa2);
                pb0 = fmaf(beta, ob.x, pb0); pb1 = fmaf(beta, ob.y, pb1); pb2 = fmaf(beta, ob.z, pb2);
            }
            q0 = fmaf(wa[0], pa0, q0); q0 = fmaf(wa[1], pa1, q0); q0 = fmaf(wa[2], pa2, q0);
            q1 = fmaf(wa[3], pa0, q1); q1 = fmaf(wa[4], pa1, q1); q1 = fmaf(wa[5], pa2, q1);
            q2 = fmaf(wa[6], pa0, q2); q2 = fmaf(wa[7], pa1, q2); q2 = fmaf(wa[8], pa2, q2);
            q0 = fmaf(wb[0], pb0, q0); q0 = fmaf(wb[1], pb1, q0); q0 = fmaf(wb[2], pb2, q0);
            q1 = fmaf(wb[3], pb0, q1); q1 = fmaf(wb[4], pb1, q1); q1 = fmaf(wb[5], pb2, q1);
            q2 = fmaf(wb[6], pb0, q2); q2 = fmaf(wb[7], pb1, q2); q2 = fmaf(wb[8], pb2, q2);
        }
        if (k < len) {
            const int b = __ldg(g.bcol + base + 32 * k + lane);
            const float *vk = v + (size_t)32 * 9 * k;
            float w[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) w[i] = __ldg(vk + 32 * i);
            const float4 z = z4[b];
            float p0 = z.x, p1 = z.y, p2 = z.z;
            if (!first) {
                const float4 po = p4[b];
                p0 = fmaf(beta, po.x, p0); p1 = fmaf(beta, po.y, p1); p2 = fmaf(beta, po.z, p2);
            }
            q0 = fmaf(w[0], p0, q0); q0 = fmaf(w[1], p1, q0); q0 = fmaf(w[2], p2, q0);
            q1 = fmaf(w[3], p0, q1); q1 = fmaf(w[4], p1, q1); q1 = fmaf(w[5], p2, q1);
            q2 = fmaf(w[6], p0, q2); q2 = fmaf(w[7], p1, q2); q2 = fmaf(w[8], p2, q2);
        }
    }
    for (int o = 1; o < tpn; o <<= 1) {
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
        q2 += __shfl_xor_sync(0xffffffffu, q2, o);
    }
}

template <class A>
__device__ __forceinline__ void spmv_row_z(const A &g, const float4 *z4, const float4 *p4, float beta, bool first,
                                           int a, int sub, bool valid, float &q0, float &q1, float &q2) {
    q0 = 0.f; q1 = 0.f; q2 = 0.f;
    const int tpn = g.tpn;
    if (valid) {
        const int s = a >> 5, lane = a & 31;
        const int base = __ldg(g.slice_ptr + s);
        const int len = __ldg(g.rowlen + a);
        if (g.block3) {
            const float *v = g.val + 9 * (size_t)base + lane;
            int k = sub;
            int bn = (k < len) ? __ldg(g.bcol + base + 32 * k + lane) : 0;
#pragma unroll 1
            for (; k < len; k += tpn) {
                const int b = bn;
                if (k + tpn < len) bn = __ldg(g.bcol + base + 32 * (k + tpn) + lane);
                const float *vk = v + (size_t)32 * 9 * k;
                const float v0 = __ldg(vk), v1 = __ldg(vk + 32), v2 = __ldg(vk + 64), v3 = __ldg(vk + 96),
                            v4 = __ldg(vk + 128), v5 = __ldg(vk + 160), v6 = __ldg(vk + 192), v7 = __ldg(vk + 224),
                            v8 = __ldg(vk + 256);
                const float4 z = z4[b];
                float p0 = z.x, p1 = z.y, p2 = z.z;
                if (!first) {
                    const float4 po = p4[b];
                    p0 = fmaf(beta, po.x, p0); p1 = fmaf(beta, po.y, p1); p2 = fmaf(beta, po.z, p2);
                }
                q0 = fmaf(v0, p0, q0); q0 = fmaf(v1, p1, q0); q0 = fmaf(v2, p2, q0);
                q1 = fmaf(v3, p0, q1); q1 = fmaf(v4, p1, q1); q1 = fmaf(v5, p2, q1);
                q2 = fmaf(v6, p0, q2); q2 = fmaf(v7, p1, q2); q2 = fmaf(v8, p2, q2);
            }
        } else {
            const float *v = g.val + base + lane;
            for (int k = sub; k < len; k += tpn) {
                const int b = __ldg(g.bcol + base + 32 * k + lane);
                const float m = __ldg(v + 32 * k);
                const float4 z = z4[b];
                float p0 = z.x, p1 = z.y, p2 = z.z;
                if (!first) {
                    const float4 po = p4[b];
                    p0 = fmaf(beta, po.x, p0); p1 = fmaf(beta, po.y, p1); p2 = fmaf(beta, po.z, p2);
                }
                q0 = fmaf(m, p0, q0);
                q1 = fmaf(m, p1, q1);
                q2 = fmaf(m, p2, q2);
            }
        }
    }
    for (int o = 1; o < tpn; o <<= 1) {
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
        q2 += __shfl_xor_sync(0xffffffffu, q2, o);
    }
}

// Bytes of dynamic shared memory cg_mixed_own_kernel needs for npb owned rows: x, r, q, p, D^{-1}, D, d.
constexpr int OWN_FIELDS = 21;
__host__ __device__ constexpr size_t own_smem_bytes(int npb) { return (size_t)OWN_FIELDS * npb * sizeof(float); }

// The mixed CG of cg_mixed_kernel with each block owning a fixed run of npb rows: the rows' x, r, q, p,
// D^{-1}, D and offsets stay in shared memory for the whole solve, the block computes its own rows' SpMV,
// and only what other blocks read goes to global memory: z = D^{-1} r (in the q buffer) and the search
// direction (double-buffered). The arithmetic is the same as cg_mixed_kernel's: p = z + beta p_old is
// formed identically by the owner and by every block that reads row b as a neighbour.
template <class R>
__global__ void __launch_bounds__(1024, 1) cg_mixed_own_kernel(const __grid_constant__ CgArgs<R> g) {
    static_assert(sizeof(R) == sizeof(float), "the owned-rows CG is the mixed path's");
    extern __shared__ float sn[];
    __shared__ float smemf[MIXED_A_NP * 32];
    __shared__ double s_sc[MIXED_GATHER_NP];
    __shared__ double s_A6[36];
    __shared__ float s_alpha, s_beta, s_tau[3], s_Om[3];
    __shared__ double s_delta;
    __shared__ int s_conv;
    DevStatus *st = g.st;
    if (st->abort) return;
    const bool defl = g.nmodes > 0;
    FFEA_PHASES_BEGIN(tm);
    float2 *partials = reinterpret_cast<float2 *>(g.partials);
    const int npb = g.npb, a0 = blockIdx.x * npb;
    const int nloc = max(0, min(npb, g.N - a0));
    float *sx = sn, *sr = sn + 3 * npb, *sq = sn + 6 * npb, *sp = sn + 9 * npb, *sdi = sn + 12 * npb,
          *sdg = sn + 15 * npb, *sd = sn + 18 * npb;
    float4 *z4 = reinterpret_cast<float4 *>(g.q);
    grid_sum_df8<MIXED_GATHER_NP>(reinterpret_cast<const float2 *>(g.init_partials), g.init_stride, g.n_init, s_sc);
    const double f2 = s_sc[0];
    mixed_setup(g, s_sc, s_A6, s_tau, s_Om, &s_beta, &s_conv);
    float acc0[1] = {0.f};
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
        const int a = a0 + l;
        float r0 = g.r[4 * a], r1 = g.r[4 * a + 1], r2 = g.r[4 * a + 2];
        const float i0 = g.dinv[4 * a], i1 = g.dinv[4 * a + 1], i2 = g.dinv[4 * a + 2];
        if (defl) {
            const float4 d = g.dpos[a];
            const float D0 = g.diag[4 * a], D1 = g.diag[4 * a + 1], D2 = g.diag[4 * a + 2];
            r0 -= D0 * (s_tau[0] + (s_Om[1] * d.z - s_Om[2] * d.y));
            r1 -= D1 * (s_tau[1] + (s_Om[2] * d.x - s_Om[0] * d.z));
            r2 -= D2 * (s_tau[2] + (s_Om[0] * d.y - s_Om[1] * d.x));
            sdg[l] = D0; sdg[npb + l] = D1; sdg[2 * npb + l] = D2;
            sd[l] = d.x; sd[npb + l] = d.y; sd[2 * npb + l] = d.z;
        }
        sr[l] = r0; sr[npb + l] = r1; sr[2 * npb + l] = r2;
        sdi[l] = i0; sdi[npb + l] = i1; sdi[2 * npb + l] = i2;
        sx[l] = 0.f; sx[npb + l] = 0.f; sx[2 * npb + l] = 0.f;
        const float z0 = i0 * r0, z1 = i1 * r1, z2 = i2 * r2;
        z4[a] = make_float4(z0, z1, z2, 0.f);
        acc0[0] += r0 * z0 + r1 * z1 + r2 * z2;
    }
    const int row0 = MIXED_A_NP + MIXED_B_NP;
    block_reduce_store<1>(acc0, smemf, partials, g.stride, row0);
    unsigned int bar_ep = 0;  // grid barriers passed
    bool ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep);
    if (ok) {
        grid_sum_df8<1>(partials + row0 * g.stride, 0, gridDim.x, s_sc);
        if (threadIdx.x == 0) s_delta = s_sc[0];
        __syncthreads();
    }
    const float4 *pold = reinterpret_cast<const float4 *>(g.pbuf0);
    float4 *pnew = reinterpret_cast<float4 *>(g.pbuf1);
    const int tpn = g.tpn, gpb = blockDim.x / tpn, grp = threadIdx.x / tpn, sub = threadIdx.x % tpn;
    const int npass = (nloc + gpb - 1) / gpb;
    FFEA_MARK(g, tm, 0);
    int it = 0;
    // a zero force (a blob exactly at rest without noise) has the solution x = 0: no iteration
    if (f2 == 0.0 && threadIdx.x == 0) s_conv = 1;
    for (; ok && it < g.imax && f2 != 0.0; ++it) {
        const bool first = it == 0;
        const float beta = s_beta;
        // phase A: q = V p over the block's rows (p formed on the fly); p.q; moments of D p
        float acc[MIXED_A_NP];
#pragma unroll
        for (int i = 0; i < MIXED_A_NP; ++i) acc[i] = 0.f;
        for (int ps = 0; ps < npass; ++ps) {
            const int l = ps * gpb + grp;
            const bool valid = l < nloc;
            float q0, q1, q2;
            if (g.block3) spmv_row_z2(g, z4, pold, beta, first, a0 + l, sub, valid, q0, q1, q2);
            else spmv_row_z(g, z4, pold, beta, first, a0 + l, sub, valid, q0, q1, q2);
            if (!valid || sub != 0) continue;
            const float z0 = sdi[l] * sr[l], z1 = sdi[npb + l] * sr[npb + l], z2 = sdi[2 * npb + l] * sr[2 * npb + l];
            float p0 = z0, p1 = z1, p2 = z2;
            if (!first) {
                p0 = fmaf(beta, sp[l], z0); p1 = fmaf(beta, sp[npb + l], z1); p2 = fmaf(beta, sp[2 * npb + l], z2);
            }
            sp[l] = p0; sp[npb + l] = p1; sp[2 * npb + l] = p2;
            sq[l] = q0; sq[npb + l] = q1; sq[2 * npb + l] = q2;
            pnew[a0 + l] = make_float4(p0, p1, p2, 0.f);
            acc[0] += p0 * q0 + p1 * q1 + p2 * q2;
            if (defl) {
                const float dx = sd[l], dy = sd[npb + l], dz = sd[2 * npb + l];
                const float e0 = sdg[l] * p0, e1 = sdg[npb + l] * p1, e2 = sdg[2 * npb + l] * p2;
                acc[1] += e0; acc[2] += e1; acc[3] += e2;
                acc[4] += dy * e2 - dz * e1;
                acc[5] += dz * e0 - dx * e2;
                acc[6] += dx * e1 - dy * e0;
            }
        }
        FFEA_MARK(g, tm, 1);
        block_reduce_store<MIXED_A_NP>(acc, smemf, partials, g.stride, 0);
        FFEA_MARK(g, tm, 2);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 3);
        grid_sum_df8<MIXED_A_NP>(partials, g.stride, gridDim.x, s_sc);
        if (threadIdx.x < 32) {
            const int ln = threadIdx.x;
            double tO = 0.0;
            if (defl && ln < 6) {
#pragma unroll
                for (int qq = 0; qq < 6; ++qq) tO += s_A6[6 * ln + qq] * s_sc[1 + qq];
            }
            double prod = (ln < 6) ? tO * s_sc[1 + ln] : 0.0;
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) prod += __shfl_xor_sync(0xffffffffu, prod, o);
            if (ln < 6) {
                if (ln < 3) s_tau[ln] = (float)tO; else s_Om[ln - 3] = (float)tO;
            }
            if (ln == 0) s_alpha = (float)s_delta / (float)(s_sc[0] + prod);
        }
        __syncthreads();
        FFEA_MARK(g, tm, 4);
        const float alpha = s_alpha;
        const float t0 = s_tau[0], t1 = s_tau[1], t2 = s_tau[2], O0 = s_Om[0], O1 = s_Om[1], O2 = s_Om[2];
        // phase B: x += alpha p ; r -= alpha (q + D (tau + Omega x d)) ; z = D^{-1} r ; r.r ; r.z
        float acc2[MIXED_B_NP] = {0.f, 0.f};
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            float p[3], qv[3], rv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                p[c] = sp[c * npb + l];
                qv[c] = sq[c * npb + l];
                sx[c * npb + l] += alpha * p[c];
            }
            if (defl) {
                const float dx = sd[l], dy = sd[npb + l], dz = sd[2 * npb + l];
                qv[0] += sdg[l] * (t0 + (O1 * dz - O2 * dy));
                qv[1] += sdg[npb + l] * (t1 + (O2 * dx - O0 * dz));
                qv[2] += sdg[2 * npb + l] * (t2 + (O0 * dy - O1 * dx));
            }
            float z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                rv[c] = sr[c * npb + l] - alpha * qv[c];
                sr[c * npb + l] = rv[c];
                z[c] = sdi[c * npb + l] * rv[c];
            }
            z4[a0 + l] = make_float4(z[0], z[1], z[2], 0.f);
            acc2[0] += rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
            acc2[1] += rv[0] * z[0] + rv[1] * z[1] + rv[2] * z[2];
        }
        FFEA_MARK(g, tm, 5);
        block_reduce_store<MIXED_B_NP>(acc2, smemf, partials, g.stride, MIXED_A_NP);
        FFEA_MARK(g, tm, 6);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 7);
        grid_sum_df8<MIXED_B_NP>(partials + MIXED_A_NP * g.stride, g.stride, gridDim.x, s_sc);
        if (threadIdx.x == 0) {
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
        const float4 *t = pold; pold = pnew; pnew = const_cast<float4 *>(t);
    }
    // the solution (and residual) back to global memory
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

// The first kc 3x3 blocks of each owned row of cg_mixed_sr_kernel, kept in shared memory for the whole solve:
// values at cv[(9 k + c) S + l], block columns at cc[k S + l] (l the row's index in the block). S is the
// block's row count padded to S = 32 / tpn (mod 32), so that the tpn lanes of a row, which read blocks k, k + 1,
// ..., k + tpn - 1 of the rows of one warp, fall on distinct banks.
struct SrCache {
    const float *cv;
    const int *cc;
    int kc, S;
};

__host__ __device__ inline int sr_cache_stride(int npb, int tpn) {
    const int r = tpn > 1 ? 32 / tpn : 0;
    int S = npb;
    while ((S & 31) != r) ++S;
    return S;
}

#define FFEA_W_FMA(WV, ZV)                                                                   \
    w0 = fmaf(WV[0], ZV.x, w0); w0 = fmaf(WV[1], ZV.y, w0); w0 = fmaf(WV[2], ZV.z, w0);        \
    w1 = fmaf(WV[3], ZV.x, w1); w1 = fmaf(WV[4], ZV.y, w1); w1 = fmaf(WV[5], ZV.z, w1);        \
    w2 = fmaf(WV[6], ZV.x, w2); w2 = fmaf(WV[7], ZV.y, w2); w2 = fmaf(WV[8], ZV.z, w2)

// Row a of w = V z for cg_mixed_sr_kernel: the preconditioned residual of neighbour b read as one float4.
// Each lane takes blocks k = sub, sub + tpn, ... in order: first those held in shared memory (k < kc), then
// the rest from the matrix in global memory, two per trip; the products are summed in block order either way,
// so the row does not depend on kc.
template <class A>
__device__ __forceinline__ void spmv_row_w(const A &g, const SrCache &c, const float4 *z4, int a, int l, int sub,
                                           bool valid, float &w0, float &w1, float &w2) {
    w0 = 0.f; w1 = 0.f; w2 = 0.f;
    const int tpn = g.tpn;
    if (valid) {
        const int s = a >> 5, lane = a & 31;
        const int base = __ldg(g.slice_ptr + s);
        const int len = __ldg(g.rowlen + a);
        const int kcl = min(c.kc, len);
        int k = sub;
#pragma unroll 1
        for (; k < kcl; k += tpn) {
            float wk[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) wk[i] = c.cv[(9 * k + i) * c.S + l];
            const float4 z = z4[c.cc[k * c.S + l]];
            FFEA_W_FMA(wk, z);
        }
        const float *v = g.val + 9 * (size_t)base + lane;
#pragma unroll 1
        for (; k + tpn < len; k += 2 * tpn) {
            const int ba = __ldg(g.bcol + base + 32 * k + lane), bb = __ldg(g.bcol + base + 32 * (k + tpn) + lane);
            const float *va = v + (size_t)32 * 9 * k, *vb = v + (size_t)32 * 9 * (k + tpn);
            float wa[9], wb[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                wa[i] = __ldg(va + 32 * i);
                wb[i] = __ldg(vb + 32 * i);
            }
            const float4 za = z4[ba], zb = z4[bb];
            FFEA_W_FMA(wa, za);
            FFEA_W_FMA(wb, zb);
        }
        if (k < len) {
            const int b = __ldg(g.bcol + base + 32 * k + lane);
            const float *vk = v + (size_t)32 * 9 * k;
            float wk[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) wk[i] = __ldg(vk + 32 * i);
            const float4 z = z4[b];
            FFEA_W_FMA(wk, z);
        }
    }
    for (int o = 1; o < tpn; o <<= 1) {
        w0 += __shfl_xor_sync(0xffffffffu, w0, o);
        w1 += __shfl_xor_sync(0xffffffffu, w1, o);
        w2 += __shfl_xor_sync(0xffffffffu, w2, o);
    }
}
#undef FFEA_W_FMA

// Bytes of dynamic shared memory cg_mixed_sr_kernel needs for npb owned rows: x, r, p, q, w, D^{-1}, D, d, and
// with a polynomial preconditioner u (the preconditioned residual) and the Chebyshev correction.
constexpr int SR_FIELDS = 24;
constexpr int SR_FIELDS_POLY = 30;
__host__ __device__ constexpr size_t sr_smem_bytes(int npb, int poly) {
    return (size_t)(poly > 0 ? SR_FIELDS_POLY : SR_FIELDS) * npb * sizeof(float);
}
// ... plus the matrix cache of kc blocks per row at stride S: nine values and a column each
constexpr int SR_CACHE_BYTES_PER_BLOCK = 10 * 4;
__host__ __device__ constexpr size_t sr_cache_bytes(int kc, int S) {
    return (size_t)SR_CACHE_BYTES_PER_BLOCK * kc * S;
}

// The Chebyshev preconditioner: degrees 2, 4, 6 and 8 (even degrees keep it positive definite whatever the
// estimate of lambda_max); the interval is [lambda_max / cheb_ratio(d), lambda_max]; the estimate comes from the
// Lanczos matrix of the first CHEB_REC iterations of a Jacobi-preconditioned solve. State (CHEB_STATE doubles):
// [0] the estimate (0: not yet known, -1: Jacobi kept), [1, 1 + CHEB_REC) step lengths, then as many direction
// coefficients, then [CHEB_KJ] the iterations of the Jacobi solve while the first polynomial solve (the trial)
// is pending.
constexpr int CHEB_MAX = 8;
constexpr int CHEB_REC = 64;
// the interval's width: degrees 4 and up gain from a wider one (40^3 Kuhn cube, degree 4, CG per step: ratio 30
// 4.24 ms, 60 4.10, 120 4.04, 250 4.06), degree 2 hardly (30 4.17, 60 4.14, 120 4.17 ms)
__host__ __device__ constexpr double cheb_ratio(int degree) { return degree > 2 ? 120.0 : 30.0; }
constexpr double CHEB_MARGIN = 1.05;
constexpr int CHEB_KJ = 1 + 2 * CHEB_REC;
constexpr int CHEB_STATE = CHEB_KJ + 1;

// Largest eigenvalue of the Lanczos matrix of n preconditioned-CG iterations (step lengths al, direction
// coefficients be, be[0] unused): T_ii = 1/al_i + be_i/al_{i-1}, T_i,i+1 = sqrt(be_{i+1})/al_i. Bisection on the
// Sturm count of negative LDL^T pivots, between the largest diagonal entry and the Gershgorin bound. One thread.
static __device__ __noinline__ double lanczos_lambda_max(const double *al, const double *be, int n) {
    double lo = 0.0, hi = 0.0;
    for (int i = 0; i < n; ++i) {
        const double d = 1.0 / al[i] + (i > 0 ? be[i] / al[i - 1] : 0.0);
        const double el = i > 0 ? sqrt(be[i]) / al[i - 1] : 0.0, er = i + 1 < n ? sqrt(be[i + 1]) / al[i] : 0.0;
        lo = fmax(lo, d);
        hi = fmax(hi, d + el + er);
    }
    for (int it = 0; it < 48 && hi - lo > 1e-6 * hi; ++it) {
        const double x = 0.5 * (lo + hi);
        int below = 0;
        double q = 1.0;
        for (int i = 0; i < n; ++i) {
            const double d = 1.0 / al[i] + (i > 0 ? be[i] / al[i - 1] : 0.0);
            const double e2 = i > 0 ? be[i] / (al[i - 1] * al[i - 1]) : 0.0;
            q = (d - x) - (i > 0 ? e2 / q : 0.0);
            if (q == 0.0) q = -1e-300;
            below += q < 0.0;
        }
        if (below == n) hi = x; else lo = x;
    }
    return hi;
}

// The mixed CG with one reduction per iteration (the single-synchronisation rearrangement of Chronopoulos and
// Gear, 1989): the SpMV is applied to the preconditioned residual z = M^{-1} r, w = V z, and the search
// direction's product follows from q = w~ + beta q_old, p = z + beta p_old, so beta is not needed before the
// SpMV. One sweep computes w and all the dot products the step needs (r.z, r.r, z.w, z.q_old, p_old.w and the
// rigid-mode moments of D z); p.q is then formed from them in FP64:
//     p.q = z.w~ + beta (z.q_old + p_old.w~) + beta^2 p_old.q_old,    w~ = w + D Z A6 Z^T D z.
// Per iteration: one grid barrier with a reduction, and one without (the new z must be visible before the
// SpMV). Rows are owned as in cg_mixed_own_kernel. With M = D (Jacobi) the iterates are, in exact arithmetic,
// those of the other mixed CG kernels; in FP32 they agree to rounding and converge in the same number of
// iterations.
// Polynomial preconditioning (g.poly = d > 0, once lambda_max of D^{-1} V is known): M^{-1} = P_d(D^{-1} V) D^{-1},
// with 1 - lambda P_d(lambda) the Chebyshev polynomial of degree d + 1 on [lambda_max / cheb_ratio(d),
// lambda_max], scaled to 1 at 0. z is built by d steps of the Chebyshev iteration for V z = r from z = 0 (d SpMVs,
// each exchanging its input vector with the neighbour blocks only), which cut the number of iterations, and with
// it the number of grid-wide reductions, by 2.8x (d = 2) to 7.7x (d = 8) on the 40^3 Kuhn cube. The
// preconditioner is built from V without the rigid-mode shift: it is positive definite on the whole spectrum for
// even d, and maps a D-weighted rigid mode D Z c to P_d(0) Z c. The shift D Z A6 Z^T D is therefore scaled by
// 1 / P_d(0) while the polynomial applies, which puts the rigid modes' eigenvalue of M^{-1} V~ at 1, inside the
// cluster of the others (unscaled they sit at P_d(0), 15.7 for d = 4 on the 40^3 cube, which then needed 132
// iterations a step instead of 110). The scale changes the shifted operator only on the rigid modes, where the
// projected right-hand side has no component, so the solution is the same: the one with Z^T D x = 0.
template <class R>
__global__ void __launch_bounds__(1024, 1) cg_mixed_sr_kernel(const __grid_constant__ CgArgs<R> g) {
    static_assert(sizeof(R) == sizeof(float), "the single-reduction CG is the mixed path's");
    extern __shared__ float sn[];
    __shared__ float smemf[MIXED_SR_NP * 32];
    __shared__ double s_sc[MIXED_GATHER_NP];
    __shared__ double s_A6[36];
    __shared__ double s_mp[6];        // moments of D p for the current direction
    __shared__ double s_g, s_pq;      // r.z and p.q~ of the previous iteration
    __shared__ float s_alpha, s_beta, s_tau[3], s_Om[3], s_dummy;
    __shared__ float s_c1[CHEB_MAX], s_c2[CHEB_MAX], s_ith;
    __shared__ double s_shift;        // scale of the rigid-mode shift: 1 / P_d(0) with the polynomial, else 1
    __shared__ int s_conv, s_stop;
    DevStatus *st = g.st;
    if (st->abort) return;
    const bool defl = g.nmodes > 0;
    FFEA_PHASES_BEGIN(tm);
    float2 *partials = reinterpret_cast<float2 *>(g.partials);
    const int npb = g.npb, a0 = blockIdx.x * npb;
    const int nloc = max(0, min(npb, g.N - a0));
    float *sx = sn, *sr = sn + 3 * npb, *sp = sn + 6 * npb, *sq = sn + 9 * npb, *sw = sn + 12 * npb,
          *sdi = sn + 15 * npb, *sdg = sn + 18 * npb, *sd = sn + 21 * npb;
    // polynomial preconditioner: u = M^{-1} r and the Chebyshev correction dd (the residual of the Chebyshev
    // iteration shares w's storage: w is dead between the update and the next SpMV)
    float *su = sn + 24 * npb, *sdd = sn + 27 * npb;
    // the matrix cache after the row fields, filled once for the solve
    SrCache mc;
    mc.kc = g.kc;
    mc.S = g.kc > 0 ? sr_cache_stride(npb, g.tpn) : 0;
    {
        float *cv = sn + (g.poly > 0 ? SR_FIELDS_POLY : SR_FIELDS) * npb;
        int *cc = reinterpret_cast<int *>(cv + 9 * (size_t)mc.kc * mc.S);
        for (int t = threadIdx.x; t < mc.kc * nloc; t += blockDim.x) {
            const int k = t / nloc, l = t - k * nloc, a = a0 + l;
            if (k >= __ldg(g.rowlen + a)) continue;
            const int base = __ldg(g.slice_ptr + (a >> 5)), lane = a & 31;
            const float *vk = g.val + 9 * (size_t)base + lane + (size_t)32 * 9 * k;
#pragma unroll
            for (int i = 0; i < 9; ++i) cv[(9 * k + i) * mc.S + l] = __ldg(vk + 32 * i);
            cc[k * mc.S + l] = __ldg(g.bcol + base + 32 * k + lane);
        }
        mc.cv = cv;
        mc.cc = cc;
    }
    float4 *z4 = reinterpret_cast<float4 *>(g.q);
    float4 *const y4a = reinterpret_cast<float4 *>(g.pbuf0), *const y4b = reinterpret_cast<float4 *>(g.pbuf1);
    const int poly = g.poly;
    const double lmax = poly > 0 ? g.cheb[0] : 0.0;
    const bool cheb = lmax > 0.0;              // Chebyshev this solve
    const bool rec = poly > 0 && lmax == 0.0;  // Jacobi this solve, recording the Lanczos coefficients
    if (cheb && threadIdx.x == 0) {
        const double b = lmax, a = lmax / cheb_ratio(poly), theta = 0.5 * (b + a), delta = 0.5 * (b - a);
        const double sigma = theta / delta;
        // the same recurrence at lambda = 0, where the residual stays D^{-1} r, gives P_d(0)
        double rho = 1.0 / sigma, p0 = 1.0 / theta, d0 = p0;
        for (int j = 0; j < poly; ++j) {
            const double rn = 1.0 / (2.0 * sigma - rho);
            s_c1[j] = (float)(rn * rho);
            s_c2[j] = (float)(2.0 * rn / delta);
            d0 = rn * rho * d0 + 2.0 * rn / delta;
            p0 += d0;
            rho = rn;
        }
        s_ith = (float)(1.0 / theta);
        s_shift = 1.0 / p0;
    }
    if (!cheb && threadIdx.x == 0) s_shift = 1.0;
    grid_sum_df8<MIXED_GATHER_NP>(reinterpret_cast<const float2 *>(g.init_partials), g.init_stride, g.n_init, s_sc);
    const double f2 = s_sc[0];
    mixed_setup(g, s_sc, s_A6, s_tau, s_Om, &s_dummy, &s_conv);
    __syncthreads();
    const float ith = cheb ? s_ith : 0.f;
    const int tpn = g.tpn, gpb = blockDim.x / tpn, grp = threadIdx.x / tpn, sub = threadIdx.x % tpn;
    const int npass = (nloc + gpb - 1) / gpb;
    unsigned int ep = 0;      // publication epochs of the neighbour exchanges
    unsigned int bar_ep = 0;  // grid barriers passed
    // Chebyshev steps 1..d after step 0 published y0 = D^{-1} r / theta (in y4a) and left D^{-1} r in sw:
    // res -= D^{-1} V y, dd = c1 dd + c2 res, u += dd; each step publishes dd for the next one's SpMV (y4a and
    // y4b alternate; a neighbour has read one before it publishes the next), the last one publishes u as z
    auto cheb_steps = [&]() -> bool {
        for (int j = 1; j <= poly; ++j) {
            const float4 *yin = (j & 1) ? y4a : y4b;
            float4 *yout = j == poly ? z4 : ((j & 1) ? y4b : y4a);
            const float c1 = s_c1[j - 1], c2 = s_c2[j - 1];
            for (int ps = 0; ps < npass; ++ps) {
                const int l = ps * gpb + grp;
                const bool valid = l < nloc;
                float t[3];
                spmv_row_w(g, mc, yin, a0 + l, l, sub, valid, t[0], t[1], t[2]);
                if (!valid || sub != 0) continue;
                float o[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float res = sw[c * npb + l] - sdi[c * npb + l] * t[c];
                    sw[c * npb + l] = res;
                    const float dd = fmaf(c1, sdd[c * npb + l], c2 * res);
                    sdd[c * npb + l] = dd;
                    const float u = su[c * npb + l] + dd;
                    su[c * npb + l] = u;
                    o[c] = j < poly ? dd : u;
                }
                yout[a0 + l] = make_float4(o[0], o[1], o[2], 0.f);
            }
            if (!neighbour_sync(g, ++ep, st)) return false;
        }
        return true;
    };
    // r = f^ (projected), x = 0, p = q = 0, z = M^{-1} r published
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
        const int a = a0 + l;
        float r0 = g.r[4 * a], r1 = g.r[4 * a + 1], r2 = g.r[4 * a + 2];
        const float i0 = g.dinv[4 * a], i1 = g.dinv[4 * a + 1], i2 = g.dinv[4 * a + 2];
        if (defl) {
            const float4 d = g.dpos[a];
            const float D0 = g.diag[4 * a], D1 = g.diag[4 * a + 1], D2 = g.diag[4 * a + 2];
            r0 -= D0 * (s_tau[0] + (s_Om[1] * d.z - s_Om[2] * d.y));
            r1 -= D1 * (s_tau[1] + (s_Om[2] * d.x - s_Om[0] * d.z));
            r2 -= D2 * (s_tau[2] + (s_Om[0] * d.y - s_Om[1] * d.x));
            sdg[l] = D0; sdg[npb + l] = D1; sdg[2 * npb + l] = D2;
            sd[l] = d.x; sd[npb + l] = d.y; sd[2 * npb + l] = d.z;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            sx[c * npb + l] = 0.f;
            sp[c * npb + l] = 0.f;
            sq[c * npb + l] = 0.f;
        }
        sr[l] = r0; sr[npb + l] = r1; sr[2 * npb + l] = r2;
        sdi[l] = i0; sdi[npb + l] = i1; sdi[2 * npb + l] = i2;
        const float z0 = i0 * r0, z1 = i1 * r1, z2 = i2 * r2;
        if (cheb) {
            const float y[3] = {z0 * ith, z1 * ith, z2 * ith}, zz[3] = {z0, z1, z2};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sw[c * npb + l] = zz[c];
                su[c * npb + l] = y[c];
                sdd[c * npb + l] = y[c];
            }
            y4a[a] = make_float4(y[0], y[1], y[2], 0.f);
        } else {
            z4[a] = make_float4(z0, z1, z2, 0.f);
        }
    }
    if (threadIdx.x < 6) s_mp[threadIdx.x] = 0.0;
    if (threadIdx.x == 0) { s_g = 0.0; s_pq = 0.0; s_stop = 0; }
    // the SpMV reads z only at neighbouring blocks' rows: wait for those blocks, not the whole grid
    bool ok = neighbour_sync(g, ++ep, st);
    if (ok && cheb) ok = cheb_steps();
    FFEA_MARK(g, tm, 0);
    int k = 0;  // updates applied so far
    s_conv = 0;
    for (; ok; ++k) {
        // w = V z over the block's rows, and the iteration's dot products
        float acc[MIXED_SR_NP];
#pragma unroll
        for (int i = 0; i < MIXED_SR_NP; ++i) acc[i] = 0.f;
        for (int ps = 0; ps < npass; ++ps) {
            const int l = ps * gpb + grp;
            const bool valid = l < nloc;
            float w0, w1, w2;
            spmv_row_w(g, mc, z4, a0 + l, l, sub, valid, w0, w1, w2);
            if (!valid || sub != 0) continue;
            sw[l] = w0; sw[npb + l] = w1; sw[2 * npb + l] = w2;
            const float r0 = sr[l], r1 = sr[npb + l], r2 = sr[2 * npb + l];
            float z0, z1, z2;
            if (cheb) {
                z0 = su[l]; z1 = su[npb + l]; z2 = su[2 * npb + l];
            } else {
                z0 = sdi[l] * r0; z1 = sdi[npb + l] * r1; z2 = sdi[2 * npb + l] * r2;
            }
            acc[0] += r0 * z0 + r1 * z1 + r2 * z2;
            acc[1] += r0 * r0 + r1 * r1 + r2 * r2;
            acc[2] += z0 * w0 + z1 * w1 + z2 * w2;
            acc[3] += z0 * sq[l] + z1 * sq[npb + l] + z2 * sq[2 * npb + l];
            acc[4] += sp[l] * w0 + sp[npb + l] * w1 + sp[2 * npb + l] * w2;
            if (defl) {
                const float dx = sd[l], dy = sd[npb + l], dz = sd[2 * npb + l];
                const float e0 = sdg[l] * z0, e1 = sdg[npb + l] * z1, e2 = sdg[2 * npb + l] * z2;
                acc[5] += e0; acc[6] += e1; acc[7] += e2;
                acc[8] += dy * e2 - dz * e1;
                acc[9] += dz * e0 - dx * e2;
                acc[10] += dx * e1 - dy * e0;
            }
        }
        FFEA_MARK(g, tm, 1);
        block_reduce_store<MIXED_SR_NP>(acc, smemf, partials, g.stride, 0);
        FFEA_MARK(g, tm, 2);
        if (!(ok = grid_sync_ep(g.gb, st, g.limit_ns, bar_ep))) break;
        FFEA_MARK(g, tm, 3);
        grid_sum_df8<MIXED_SR_NP>(partials, g.stride, gridDim.x, s_sc);
        if (threadIdx.x < 32) {
            const int ln = threadIdx.x;
            // c = s A6 m(z): the rigid-mode coefficients of s D Z A6 Z^T D z, over six lanes
            double c = 0.0;
            if (defl && ln < 6) {
#pragma unroll
                for (int qq = 0; qq < 6; ++qq) c += s_A6[6 * ln + qq] * s_sc[5 + qq];
                c *= s_shift;
            }
            double mzc = (ln < 6) ? s_sc[5 + ln] * c : 0.0;   // m(z).c
            double mpc = (ln < 6) ? s_mp[ln] * c : 0.0;       // m(p_old).c
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) {
                mzc += __shfl_xor_sync(0xffffffffu, mzc, o);
                mpc += __shfl_xor_sync(0xffffffffu, mpc, o);
            }
            const double gam = s_sc[0], rr = s_sc[1];
            // |r|^2/|f|^2 < epsilon2 after an update, as NoMassCGSolver::solve tests it (a zero force: x = 0 at once)
            const bool conv = f2 == 0.0 || (k > 0 && (g.check_last || k < g.imax) && rr < g.eps2 * f2);
            if (ln == 0 && blockIdx.x == 0 && k > 0 && k - 1 < g.hist_cap) g.history[k - 1] = (f2 == 0.0) ? 0.0 : rr / f2;
            const bool stop = conv || k >= g.imax;
            // the step lengths in FP32 (as cg_mixed_kernel forms them): FP64 division is slow on this GPU
            const float beta_f = (k == 0) ? 0.f : (float)gam / (float)s_g;
            const double beta = beta_f;
            const double zw = s_sc[2] + mzc, pw = s_sc[4] + mpc;
            const double pq = zw + beta * (s_sc[3] + pw) + beta * beta * s_pq;
            if (rec && ln == 0 && blockIdx.x == 0 && !stop && k < CHEB_REC) {
                g.cheb[1 + k] = gam / pq;
                g.cheb[1 + CHEB_REC + k] = beta;
            }
            __syncwarp();
            if (ln < 6) {
                const float cf = (float)c;
                if (ln < 3) s_tau[ln] = cf; else s_Om[ln - 3] = cf;
                s_mp[ln] = s_sc[5 + ln] + beta * s_mp[ln];
            }
            if (ln == 0) {
                s_conv = conv;
                s_stop = stop;
                s_beta = beta_f;
                s_alpha = (float)gam / (float)pq;
                s_g = gam;
                s_pq = pq;
            }
        }
        __syncthreads();
        FFEA_MARK(g, tm, 4);
        if (s_stop) break;
        const float alpha = s_alpha, beta = s_beta;
        const float t0 = s_tau[0], t1 = s_tau[1], t2 = s_tau[2], O0 = s_Om[0], O1 = s_Om[1], O2 = s_Om[2];
        // p = z + beta p ; q = w~ + beta q ; x += alpha p ; r -= alpha q ; z = M^{-1} r published (Jacobi), or
        // the Chebyshev iteration's first step (polynomial)
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            const int a = a0 + l;
            float wv[3] = {sw[l], sw[npb + l], sw[2 * npb + l]};
            if (defl) {
                const float dx = sd[l], dy = sd[npb + l], dz = sd[2 * npb + l];
                wv[0] += sdg[l] * (t0 + (O1 * dz - O2 * dy));
                wv[1] += sdg[npb + l] * (t1 + (O2 * dx - O0 * dz));
                wv[2] += sdg[2 * npb + l] * (t2 + (O0 * dy - O1 * dx));
            }
            float zn[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float r = sr[c * npb + l], di = sdi[c * npb + l];
                const float zc = cheb ? su[c * npb + l] : di * r;
                const float pv = fmaf(beta, sp[c * npb + l], zc);
                const float qv = fmaf(beta, sq[c * npb + l], wv[c]);
                sp[c * npb + l] = pv;
                sq[c * npb + l] = qv;
                sx[c * npb + l] += alpha * pv;
                const float rn = r - alpha * qv;
                sr[c * npb + l] = rn;
                zn[c] = di * rn;
                if (cheb) {
                    const float y = zn[c] * ith;
                    sw[c * npb + l] = zn[c];
                    su[c * npb + l] = y;
                    sdd[c * npb + l] = y;
                    zn[c] = y;
                }
            }
            (cheb ? y4a : z4)[a] = make_float4(zn[0], zn[1], zn[2], 0.f);
        }
        FFEA_MARK(g, tm, 5);
        if (!(ok = neighbour_sync(g, ++ep, st))) break;
        FFEA_MARK(g, tm, 7);
        if (cheb && !(ok = cheb_steps())) break;
        FFEA_MARK(g, tm, 6);
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
            st->last_iters = k;
            st->total_iters += k;
            if (rec && k >= 2) {
                // the estimate of lambda_max(D^-1 V) for the next solves, from this Jacobi solve's Lanczos matrix
                const double lm = lanczos_lambda_max(g.cheb + 1, g.cheb + 1 + CHEB_REC, min(k, CHEB_REC));
                if (isfinite(lm) && lm > 0.0) {
                    g.cheb[0] = CHEB_MARGIN * lm;
                    g.cheb[CHEB_KJ] = (double)k;
                }
            } else if (cheb && g.cheb[CHEB_KJ] > 0.0) {
                // the trial: the polynomial is kept when its iterations, each costing 1 + poly * cheb_cost Jacobi
                // iterations, took less than the Jacobi solve (a well-conditioned matrix, e.g. with a large
                // Stokes drag on its diagonal, converges in a few Jacobi iterations and keeps Jacobi)
                if ((double)k * (1.0 + poly * (double)g.cheb_cost) >= g.cheb[CHEB_KJ]) g.cheb[0] = -1.0;
                g.cheb[CHEB_KJ] = 0.0;
            }
        }
    }
}

}  // namespace ffea
