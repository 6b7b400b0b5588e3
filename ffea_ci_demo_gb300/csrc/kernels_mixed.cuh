// kernels_mixed.cuh -- the mixed-precision force gather and CG solve.
//
// The viscosity matrix of a blob with no Stokes drag is singular: rigid
// translations and rotations (restricted to motions that leave every pinned
// node at rest) produce no viscous stress, so K z = 0 for them. The reference's
// FP64 CG never excites these directions far enough to matter before it
// converges; with an FP32 matrix and SpMV, rounding puts ~1e-7 of every
// product into them and the 1e-10 relative residual becomes unreachable.
// This solver therefore keeps the residual orthogonal to the rigid modes:
// every SpMV output q is replaced by q - Z G^{-1} Z^T q, which is what exact
// arithmetic would give, with Z^T q formed from the moments
// S1 = sum_a q_a and S2 = sum_a d_a x q_a (d_a = node position minus the rest
// centroid) accumulated with exact FP64 products.
//
// Precision: matrix values, SpMV, p, q, x in FP32; the residual r, its
// updates, the preconditioned residual z = D^{-1} r, every dot product and
// the projection moments in FP64. Iteration counts match the FP64 solver.
#pragma once

#include "kernels.cuh"

namespace ffea {

constexpr int MIXED_GATHER_NP = 16;  // f.f, S1_f(3), S2_f(3), sum d(3), inertia(6)
constexpr int MIXED_A_NP = 13;       // p.q, S1_q(3), S2_q(3), S1_p(3), S2_p(3)
constexpr int MIXED_B_NP = 8;        // r.r, r.z, and (diagnostics) S1_r(3), S2_r(3)
// partials rows: [0, A) phase A, [A, A+B) phase B, A+B the initial r.z. Each row is written in one phase
// and read right after the next grid barrier; no row is written again before every block has passed
// the barrier that follows its read.
constexpr int MIXED_PARTIAL_ROWS = MIXED_A_NP + MIXED_B_NP + 1;

// mixed-path gather: f (FP64) and r = f; per-node offsets d; projection moments
template <class R>
__global__ void __launch_bounds__(256) gather_mixed_kernel(GatherArgs<R> g) {
    __shared__ double smem[MIXED_GATHER_NP * 32];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a == 0 && g.gb) g.gb->count = 0u;
    double acc[MIXED_GATHER_NP];
#pragma unroll
    for (int i = 0; i < MIXED_GATHER_NP; ++i) acc[i] = 0.0;
    if (a < g.N && !g.st->abort) {
        float F0 = 0, F1 = 0, F2 = 0;
        for (int m = g.inc_ptr[a]; m < g.inc_ptr[a + 1]; ++m) {
            const int es = g.inc[m];
            const R *c = g.ef + 12 * (size_t)(es >> 2) + 3 * (es & 3);
            F0 += c[0];
            F1 += c[1];
            F2 += c[2];
        }
        if (g.drag) {
            const double dr = g.drag[a];
            F0 -= (float)(g.vx[a] * dr);
            F1 -= (float)(g.vy[a] * dr);
            F2 -= (float)(g.vz[a] * dr);
        }
        if (g.pinned[a]) { F0 = 0; F1 = 0; F2 = 0; }
        const double f0 = F0, f1 = F1, f2 = F2;
        g.f[4 * a] = f0; g.f[4 * a + 1] = f1; g.f[4 * a + 2] = f2;
        if (g.mode == 1) {
            g.x[4 * a] = F0 * g.dinv[4 * a];
            g.x[4 * a + 1] = F1 * g.dinv[4 * a + 1];
            g.x[4 * a + 2] = F2 * g.dinv[4 * a + 2];
            return;
        }
        g.r64[4 * a] = f0; g.r64[4 * a + 1] = f1; g.r64[4 * a + 2] = f2;
        const float d0 = (float)(g.px[a] - g.xc[0]), d1 = (float)(g.py[a] - g.xc[1]), d2 = (float)(g.pz[a] - g.xc[2]);
        g.dpos[a] = make_float4(d0, d1, d2, 0.f);
        const double e0 = d0, e1 = d1, e2 = d2;
        acc[0] = f0 * f0 + f1 * f1 + f2 * f2;
        acc[1] = f0; acc[2] = f1; acc[3] = f2;
        acc[4] = e1 * f2 - e2 * f1; acc[5] = e2 * f0 - e0 * f2; acc[6] = e0 * f1 - e1 * f0;
        acc[7] = e0; acc[8] = e1; acc[9] = e2;
        // sum_a (|d|^2 I - d d^T): xx, yy, zz, xy, xz, yz
        const double dd = e0 * e0 + e1 * e1 + e2 * e2;
        acc[10] = dd - e0 * e0; acc[11] = dd - e1 * e1; acc[12] = dd - e2 * e2;
        acc[13] = -e0 * e1; acc[14] = -e0 * e2; acc[15] = -e1 * e2;
    }
    if (g.mode == 1) return;
    block_sum<MIXED_GATHER_NP>(acc, smem);
    if (threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < MIXED_GATHER_NP; ++i) g.partials[i * g.stride + blockIdx.x] = acc[i];
}

// c = Ginv (T S1 + W S2); tau = T^T c; Omega = W^T c  (one thread)
template <class R>
__device__ __forceinline__ void mode_coeffs(const CgArgs<R> &g, const double *Ginv, const double S1[3],
                                            const double S2[3], double c[6], double tau[3], double Om[3]) {
    double v[6];
    for (int k = 0; k < g.nmodes; ++k) {
        const double *m = g.modes + 6 * k;
        v[k] = m[0] * S1[0] + m[1] * S1[1] + m[2] * S1[2] + m[3] * S2[0] + m[4] * S2[1] + m[5] * S2[2];
    }
    for (int j = 0; j < g.nmodes; ++j) {
        double s = 0.0;
        for (int k = 0; k < g.nmodes; ++k) s += Ginv[6 * j + k] * v[k];
        c[j] = s;
    }
    for (int i = 0; i < 3; ++i) { tau[i] = 0.0; Om[i] = 0.0; }
    for (int k = 0; k < g.nmodes; ++k) {
        const double *m = g.modes + 6 * k;
        for (int i = 0; i < 3; ++i) { tau[i] += c[k] * m[i]; Om[i] += c[k] * m[3 + i]; }
    }
}

template <class R>
__global__ void __launch_bounds__(1024, 1) cg_mixed_kernel(CgArgs<R> g) {
    __shared__ double smem[MIXED_A_NP * 32];
    __shared__ double s_Ginv[36];
    __shared__ double s_tau[3], s_Om[3], s_pq;
    DevStatus *st = g.st;
    if (st->abort) return;
    const int nthr = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const bool defl = g.nmodes > 0;
    // set-up: moments of f, Gram matrix of the modes, projected initial residual
    double gp[MIXED_GATHER_NP];
    grid_partials_sum<MIXED_GATHER_NP>(g.init_partials, g.init_stride, g.n_init, gp, smem);
    const double f2 = gp[0];
    if (threadIdx.x == 0) {
        double G[36], Ginv[36];
        const int k = g.nmodes;
        const double Nn = (double)g.N;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                const double *ti = g.modes + 6 * i, *tj = g.modes + 6 * j;
                // t_i.t_j N + t_i.(w_j x sd) + t_j.(w_i x sd) + w_i^T I w_j
                const double sd[3] = {gp[7], gp[8], gp[9]};
                auto cross_dot = [&](const double *t, const double *w) {
                    return t[0] * (w[1] * sd[2] - w[2] * sd[1]) + t[1] * (w[2] * sd[0] - w[0] * sd[2]) +
                           t[2] * (w[0] * sd[1] - w[1] * sd[0]);
                };
                const double I[9] = {gp[10], gp[13], gp[14], gp[13], gp[11], gp[15], gp[14], gp[15], gp[12]};
                double wIw = 0.0;
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q) wIw += ti[3 + p] * I[3 * p + q] * tj[3 + q];
                G[6 * i + j] = Nn * (ti[0] * tj[0] + ti[1] * tj[1] + ti[2] * tj[2]) + cross_dot(ti, tj + 3) +
                               cross_dot(tj, ti + 3) + wIw;
            }
        // Gauss-Jordan inverse of the small SPD Gram matrix
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) Ginv[6 * i + j] = (i == j) ? 1.0 : 0.0;
        for (int col = 0; col < k; ++col) {
            const double piv = G[6 * col + col];
            for (int j = 0; j < k; ++j) { G[6 * col + j] /= piv; Ginv[6 * col + j] /= piv; }
            for (int i = 0; i < k; ++i) {
                if (i == col) continue;
                const double fct = G[6 * i + col];
                for (int j = 0; j < k; ++j) { G[6 * i + j] -= fct * G[6 * col + j]; Ginv[6 * i + j] -= fct * Ginv[6 * col + j]; }
            }
        }
        for (int i = 0; i < 36; ++i) s_Ginv[i] = Ginv[i];
        double c[6], tau[3] = {0, 0, 0}, Om[3] = {0, 0, 0};
        if (defl) {
            const double S1[3] = {gp[1], gp[2], gp[3]}, S2[3] = {gp[4], gp[5], gp[6]};
            mode_coeffs(g, Ginv, S1, S2, c, tau, Om);
        }
        for (int i = 0; i < 3; ++i) { s_tau[i] = tau[i]; s_Om[i] = Om[i]; }
    }
    __syncthreads();
    double acc0[1] = {0.0};
    for (int a = tid; a < g.N; a += nthr) {
        const float4 d = g.dpos[a];
        const double e0 = d.x, e1 = d.y, e2 = d.z;
        double r0 = g.r64[4 * a], r1 = g.r64[4 * a + 1], r2 = g.r64[4 * a + 2];
        if (defl) {
            r0 -= s_tau[0] + (s_Om[1] * e2 - s_Om[2] * e1);
            r1 -= s_tau[1] + (s_Om[2] * e0 - s_Om[0] * e2);
            r2 -= s_tau[2] + (s_Om[0] * e1 - s_Om[1] * e0);
            g.r64[4 * a] = r0; g.r64[4 * a + 1] = r1; g.r64[4 * a + 2] = r2;
        }
        const double z0 = (double)g.dinv[4 * a] * r0, z1 = (double)g.dinv[4 * a + 1] * r1,
                     z2 = (double)g.dinv[4 * a + 2] * r2;
        g.p[4 * a] = (float)z0; g.p[4 * a + 1] = (float)z1; g.p[4 * a + 2] = (float)z2;
        g.x[4 * a] = 0.f; g.x[4 * a + 1] = 0.f; g.x[4 * a + 2] = 0.f;
        acc0[0] += r0 * z0 + r1 * z1 + r2 * z2;
    }
    block_sum<1>(acc0, smem);
    const int row0 = MIXED_A_NP + MIXED_B_NP;
    if (threadIdx.x == 0) g.partials[row0 * g.stride + blockIdx.x] = acc0[0];
    bool ok = grid_sync(g.gb, st, g.limit_ns);
    double delta = 0.0;
    if (ok) {
        double d0[1];
        grid_partials_sum<1>(g.partials + row0 * g.stride, 0, gridDim.x, d0, smem);
        delta = d0[0];
    }
    int it = 0;
    bool converged = false;
    for (; ok && it < g.imax; ++it) {
        // phase A: q = V p, p.q and the projection moments of q and p
        double acc[MIXED_A_NP];
#pragma unroll
        for (int i = 0; i < MIXED_A_NP; ++i) acc[i] = 0.0;
        FFEA_SPMV_LOOP(g, a, sub, valid) {
            float q0, q1, q2;
            spmv_row(g, a, sub, valid, q0, q1, q2);
            if (!valid || sub != 0) continue;
            g.q[4 * a] = q0; g.q[4 * a + 1] = q1; g.q[4 * a + 2] = q2;
            const float p0 = g.p[4 * a], p1 = g.p[4 * a + 1], p2 = g.p[4 * a + 2];
            acc[0] += (double)(p0 * q0 + p1 * q1 + p2 * q2);
            if (defl) {
                const float4 d = g.dpos[a];
                const double e0 = d.x, e1 = d.y, e2 = d.z, Q0 = q0, Q1 = q1, Q2 = q2;
                acc[1] += Q0; acc[2] += Q1; acc[3] += Q2;
                acc[4] += e1 * Q2 - e2 * Q1; acc[5] += e2 * Q0 - e0 * Q2; acc[6] += e0 * Q1 - e1 * Q0;
                acc[7] += (double)p0; acc[8] += (double)p1; acc[9] += (double)p2;
                acc[10] += (double)(d.y * p2 - d.z * p1);
                acc[11] += (double)(d.z * p0 - d.x * p2);
                acc[12] += (double)(d.x * p1 - d.y * p0);
            }
        }
        block_sum<MIXED_A_NP>(acc, smem);
        if (threadIdx.x == 0)
#pragma unroll
            for (int i = 0; i < MIXED_A_NP; ++i) g.partials[i * g.stride + blockIdx.x] = acc[i];
        if (!(ok = grid_sync(g.gb, st, g.limit_ns))) break;
        double sa[MIXED_A_NP];
        grid_partials_sum<MIXED_A_NP>(g.partials, g.stride, gridDim.x, sa, smem);
        if (threadIdx.x == 0) {
            double c[6], tau[3] = {0, 0, 0}, Om[3] = {0, 0, 0}, pq = sa[0];
            if (defl) {
                const double S1q[3] = {sa[1], sa[2], sa[3]}, S2q[3] = {sa[4], sa[5], sa[6]};
                mode_coeffs(g, s_Ginv, S1q, S2q, c, tau, Om);
                for (int k = 0; k < g.nmodes; ++k) {
                    const double *m = g.modes + 6 * k;
                    const double zp = m[0] * sa[7] + m[1] * sa[8] + m[2] * sa[9] + m[3] * sa[10] + m[4] * sa[11] +
                                      m[5] * sa[12];
                    pq -= zp * c[k];
                }
            }
            for (int i = 0; i < 3; ++i) { s_tau[i] = tau[i]; s_Om[i] = Om[i]; }
            s_pq = pq;
        }
        __syncthreads();
        const double alpha = delta / s_pq;
        const float af = (float)alpha;
        const double t0 = s_tau[0], t1 = s_tau[1], t2 = s_tau[2], O0 = s_Om[0], O1 = s_Om[1], O2 = s_Om[2];
        // phase B: x += alpha p ; r -= alpha (q - tau - Omega x d) ; r.r ; r.z
        double acc2[MIXED_B_NP] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = tid; a < g.N; a += nthr) {
#pragma unroll
            for (int c = 0; c < 3; ++c) g.x[4 * a + c] += af * g.p[4 * a + c];
            double qh0 = g.q[4 * a], qh1 = g.q[4 * a + 1], qh2 = g.q[4 * a + 2];
            if (defl) {
                const float4 d = g.dpos[a];
                const double e0 = d.x, e1 = d.y, e2 = d.z;
                qh0 -= t0 + (O1 * e2 - O2 * e1);
                qh1 -= t1 + (O2 * e0 - O0 * e2);
                qh2 -= t2 + (O0 * e1 - O1 * e0);
            }
            const double r0 = g.r64[4 * a] - alpha * qh0, r1 = g.r64[4 * a + 1] - alpha * qh1,
                         r2 = g.r64[4 * a + 2] - alpha * qh2;
            g.r64[4 * a] = r0; g.r64[4 * a + 1] = r1; g.r64[4 * a + 2] = r2;
            const double z0 = (double)g.dinv[4 * a] * r0, z1 = (double)g.dinv[4 * a + 1] * r1,
                         z2 = (double)g.dinv[4 * a + 2] * r2;
            acc2[0] += r0 * r0 + r1 * r1 + r2 * r2;
            acc2[1] += r0 * z0 + r1 * z1 + r2 * z2;
            if (g.debug & 2) {
                const float4 d = g.dpos[a];
                const double e0 = d.x, e1 = d.y, e2 = d.z;
                acc2[2] += r0; acc2[3] += r1; acc2[4] += r2;
                acc2[5] += e1 * r2 - e2 * r1; acc2[6] += e2 * r0 - e0 * r2; acc2[7] += e0 * r1 - e1 * r0;
            }
        }
        block_sum<MIXED_B_NP>(acc2, smem);
        if (threadIdx.x == 0)
            for (int i = 0; i < MIXED_B_NP; ++i) g.partials[(MIXED_A_NP + i) * g.stride + blockIdx.x] = acc2[i];
        if (!(ok = grid_sync(g.gb, st, g.limit_ns))) break;
        double rz[MIXED_B_NP];
        grid_partials_sum<MIXED_B_NP>(g.partials + MIXED_A_NP * g.stride, g.stride, gridDim.x, rz, smem);
        const double res2 = (f2 == 0.0) ? 0.0 : rz[0] / f2;
        if ((g.debug & 2) && blockIdx.x == 0 && threadIdx.x == 0 && it < g.hist_cap && defl) {
            double c[6], tau[3], Om[3];
            const double S1r[3] = {rz[2], rz[3], rz[4]}, S2r[3] = {rz[5], rz[6], rz[7]};
            mode_coeffs(g, s_Ginv, S1r, S2r, c, tau, Om);
            double v = 0.0;  // (Z^T r)^T G^-1 (Z^T r) / f2
            for (int k = 0; k < g.nmodes; ++k) {
                const double *m = g.modes + 6 * k;
                v += c[k] * (m[0] * S1r[0] + m[1] * S1r[1] + m[2] * S1r[2] + m[3] * S2r[0] + m[4] * S2r[1] + m[5] * S2r[2]);
            }
            g.history[it] = v / f2;  // replaces res2 in the history when debugging
        }
        if (blockIdx.x == 0 && threadIdx.x == 0 && it < g.hist_cap && !(g.debug & 2)) g.history[it] = res2;
        if ((g.check_last || it + 1 < g.imax) && res2 < g.eps2) {
            converged = true;
            ++it;
            break;
        }
        const double delta_old = delta;
        delta = rz[1];
        const float beta = (float)(delta / delta_old);
        // phase C: p = beta p + z
        for (int a = tid; a < g.N; a += nthr) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                g.p[4 * a + c] = beta * g.p[4 * a + c] + (float)((double)g.dinv[4 * a + c] * g.r64[4 * a + c]);
        }
        if (!(ok = grid_sync(g.gb, st, g.limit_ns))) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!ok) {
            st->abort = 1;
        } else if (!converged) {
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
