// kernels_adjoint.cuh -- reverse-mode derivative of the NoMass blob step.
//
// One NoMass step is x_{n+1} = x_n + dt v_n with v_n = S(x_n) f(x_n, theta, xi_n): V(x_n) v_n = f
// (src/NoMassCGSolver.cpp:156-188, src/Blob.cpp:3249-3279), where S is the map the Jacobi-PCG
// realises from x = 0: the solution of V v = f that is D-orthogonal to the rigid modes Z (Z^T D v = 0,
// D = diag V). S is symmetric (S = V~^{-1} - Z G^{-1} Z^T with V~ = V + D Z G^{-1} Z^T D), so the
// adjoint solve is the forward solve applied to dt lambda_{n+1}:
//     mu = S (dt lambda_{n+1}),    rho = G^{-1} Z^T (dt lambda_{n+1})
// and, with r_e(x, theta) = f_e - V_e v_e the element residual at fixed v,
//     lambda_n   = lambda_{n+1} + sum_e d/dx [mu_e^T r_e - sum_a (Z_a rho) . (D_a v_a)]
//     dL/dtheta += sum_e d/dtheta [ same ]
// The second term is the derivative of the constraint Z^T D v = 0: moving the nodes changes both
// the rigid modes (through the node offsets) and the diagonal D.
//
// Per element, mu_e^T r_e = -vol <grad mu, T> with T = S_el + N + sigma_v: the elastic stress S_el,
// the fluctuating stress N (frozen draws) and the viscous stress sigma_v = B tr(L) I + A (L + L^T)
// of the forward velocity gradient L (tetra_element_linear, src/tetra_element_linear.cpp:298-443).
// elem_vjp_kernel differentiates it by hand with respect to the edge matrix J and to G, E, A, B.
#pragma once

#include "kernels_mixed.cuh"

namespace ffea {

constexpr int ADJ_MOMENTS = MIXED_GATHER_NP;  // |F|^2, S1(3), S2(3), M (21)

template <class R>
struct AdjGatherArgs {
    int N;
    double dt;
    const double *lam;    // 4 per node: lambda_{n+1}
    const int *pinned;
    const double *px, *py, *pz;
    double xc[3];
    const R *dinv, *diag; // diag: mixed path only (FP64 path: D = 1 / dinv)
    double *f;
    R *r, *x;
    float4 *dpos;         // mixed path
    double *partials_d;   // FP64 path: ADJ_MOMENTS rows of per-block sums
    float2 *partials_f;   // mixed path: the same as double-float pairs (the layout cg_mixed_kernel reads)
    int stride;
    GridBarrier *gb;
    const DevStatus *st;
};

// right-hand side dt lambda (pinned rows zero, as the gather zeroes pinned forces), r = rhs, x = 0,
// and the per-block moments of the rigid-mode set-up (gather_mixed_kernel's set, summed in FP64)
template <class R>
__global__ void __launch_bounds__(256) adj_gather_kernel(AdjGatherArgs<R> g) {
    __shared__ double smem[ADJ_MOMENTS * 32];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a == 0 && g.gb) g.gb->count = 0u;
    double acc[ADJ_MOMENTS];
#pragma unroll
    for (int i = 0; i < ADJ_MOMENTS; ++i) acc[i] = 0.0;
    if (a < g.N && !g.st->abort) {
        double F[3];
        for (int c = 0; c < 3; ++c) F[c] = g.pinned[a] ? 0.0 : g.dt * g.lam[4 * (size_t)a + c];
        const double d[3] = {g.px[a] - g.xc[0], g.py[a] - g.xc[1], g.pz[a] - g.xc[2]};
        double D[3];
        for (int c = 0; c < 3; ++c) {
            g.f[4 * (size_t)a + c] = F[c];
            g.r[4 * (size_t)a + c] = (R)F[c];
            g.x[4 * (size_t)a + c] = (R)0;
            D[c] = g.diag ? (double)g.diag[4 * (size_t)a + c] : 1.0 / (double)g.dinv[4 * (size_t)a + c];
        }
        if (g.dpos) g.dpos[a] = make_float4((float)d[0], (float)d[1], (float)d[2], 0.f);
        acc[0] = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
        acc[1] = F[0]; acc[2] = F[1]; acc[3] = F[2];
        acc[4] = d[1] * F[2] - d[2] * F[1]; acc[5] = d[2] * F[0] - d[0] * F[2]; acc[6] = d[0] * F[1] - d[1] * F[0];
        const double phi[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                  {0, -d[2], d[1]}, {d[2], 0, -d[0]}, {-d[1], d[0], 0}};
        int k = 7;
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j, ++k)
                acc[k] = phi[i][0] * D[0] * phi[j][0] + phi[i][1] * D[1] * phi[j][1] + phi[i][2] * D[2] * phi[j][2];
    }
    block_sum<ADJ_MOMENTS>(acc, smem);
    if (threadIdx.x == 0) {
        for (int i = 0; i < ADJ_MOMENTS; ++i) {
            if (g.partials_d) g.partials_d[i * g.stride + blockIdx.x] = acc[i];
            if (g.partials_f) {
                const float hi = (float)acc[i];
                g.partials_f[i * g.stride + blockIdx.x] = make_float2(hi, (float)(acc[i] - (double)hi));
            }
        }
    }
}

// rigid-mode coefficients of rho = G^{-1} Z^T rhs: coef = (tau, Omega) with Z rho at node a equal to
// tau + Omega x d_a. One block; `modes` as for the mixed-path set-up.
struct AdjModesArgs {
    const double *partials_d;
    const float2 *partials_f;
    int stride, nb;
    int nmodes;
    double modes[36];
    double *coef;  // 6
};

template <class R>  // R: the instantiating path (the kernel itself is precision-independent)
__global__ void __launch_bounds__(256) adj_modes_kernel(const __grid_constant__ AdjModesArgs g) {
    __shared__ double s_sc[ADJ_MOMENTS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wid; i < ADJ_MOMENTS; i += nw) {
        double t = 0.0;
        for (int b = lane; b < g.nb; b += 32)
            t += g.partials_d ? g.partials_d[i * g.stride + b]
                              : (double)g.partials_f[i * g.stride + b].x + (double)g.partials_f[i * g.stride + b].y;
        t = warp_sum(t);
        if (lane == 0) s_sc[i] = t;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int k = g.nmodes;
    double out[6] = {0, 0, 0, 0, 0, 0};
    if (k > 0) {
        double M[6][6];
        int idx = 7;
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j, ++idx) M[i][j] = M[j][i] = s_sc[idx];
        double G[36], Gi[36];
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                double sum = 0.0;
                for (int p = 0; p < 6; ++p)
                    for (int q = 0; q < 6; ++q) sum += g.modes[6 * i + p] * M[p][q] * g.modes[6 * j + q];
                G[6 * i + j] = sum;
                Gi[6 * i + j] = (i == j) ? 1.0 : 0.0;
            }
        for (int col = 0; col < k; ++col) {
            const double piv = G[6 * col + col];
            for (int j = 0; j < k; ++j) { G[6 * col + j] /= piv; Gi[6 * col + j] /= piv; }
            for (int i = 0; i < k; ++i) {
                if (i == col) continue;
                const double fct = G[6 * i + col];
                for (int j = 0; j < k; ++j) { G[6 * i + j] -= fct * G[6 * col + j]; Gi[6 * i + j] -= fct * Gi[6 * col + j]; }
            }
        }
        double v[6];
        for (int i = 0; i < k; ++i) {
            const double *m = g.modes + 6 * i;
            v[i] = m[0] * s_sc[1] + m[1] * s_sc[2] + m[2] * s_sc[3] + m[3] * s_sc[4] + m[4] * s_sc[5] + m[5] * s_sc[6];
        }
        for (int i = 0; i < k; ++i) {
            double c = 0.0;
            for (int j = 0; j < k; ++j) c += Gi[6 * i + j] * v[j];
            for (int t = 0; t < 6; ++t) out[t] += c * g.modes[6 * i + t];
        }
    }
    for (int t = 0; t < 6; ++t) g.coef[t] = out[t];
}

// FP64 path: project the right-hand side, r = rhs - D Z rho (the plain CG needs a consistent system),
// and the opening sums |r|^2, r.z of cg_kernel
template <class R>
struct AdjApplyArgs {
    int N;
    const double *px, *py, *pz;
    double xc[3];
    const double *coef;
    const R *dinv;
    R *r;
    double *f;
    double *partials;  // 2 rows
    int stride;
    const DevStatus *st;
};

template <class R>
__global__ void __launch_bounds__(256) adj_apply_kernel(AdjApplyArgs<R> g) {
    __shared__ double smem[64];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[2] = {0.0, 0.0};
    if (a < g.N && !g.st->abort) {
        const double d[3] = {g.px[a] - g.xc[0], g.py[a] - g.xc[1], g.pz[a] - g.xc[2]};
        const double *t = g.coef, *O = g.coef + 3;
        const double rv[3] = {t[0] + (O[1] * d[2] - O[2] * d[1]), t[1] + (O[2] * d[0] - O[0] * d[2]),
                              t[2] + (O[0] * d[1] - O[1] * d[0])};
        for (int c = 0; c < 3; ++c) {
            const double di = (double)g.dinv[4 * (size_t)a + c];
            const double rc = g.f[4 * (size_t)a + c] - rv[c] / di;
            g.r[4 * (size_t)a + c] = (R)rc;
            g.f[4 * (size_t)a + c] = rc;
            acc[0] += rc * rc;
            acc[1] += rc * (di * rc);
        }
    }
    block_sum<2>(acc, smem);
    if (threadIdx.x == 0) {
        g.partials[blockIdx.x] = acc[0];
        g.partials[g.stride + blockIdx.x] = acc[1];
    }
}

// element VJP: d/dx and d/dtheta of s_e = mu_e^T r_e - sum_a (Z_a rho) . (D_a^e v_a), D^e the element's
// share of diag V
template <class R>
struct AdjElemArgs {
    int T, calc_noise;
    double kT, dt;
    const int4 *tet;
    const double *px, *py, *pz;
    const R *jinv, *G, *E, *A, *B, *vol0;
    const uint32_t *rng_state;
    const MrgJump *chunk_jump, *lane_jump;
    const R *mu;         // 4 per node: adjoint solution
    const R *v;          // 4 per node: forward velocity of the step
    int nmodes;
    double xc[3];
    const double *coef;  // (tau, Omega) of Z rho
    double *eg;          // 12 per element: gradient of s_e with respect to the 4 vertex positions
    double *gtheta;      // 4 per element, accumulated: d/dG, d/dE, d/dA, d/dB
    const DevStatus *st;
};

template <class R>
__global__ void __launch_bounds__(128) elem_vjp_kernel(AdjElemArgs<R> g) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.T || g.st->abort) return;
    const int4 t = g.tet[e];
    const int nd[4] = {t.x, t.y, t.z, t.w};
    double X[4][3];
    for (int a = 0; a < 4; ++a) { X[a][0] = g.px[nd[a]]; X[a][1] = g.py[nd[a]]; X[a][2] = g.pz[nd[a]]; }
    double J[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) J[i][j] = X[i + 1][j] - X[0][j];
    // K = J^{-1} by cofactors (calc_shape_function_derivatives_and_volume :222-292)
    double K[3][3];
    K[0][0] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    K[0][1] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    K[0][2] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    K[1][0] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
    K[1][1] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
    K[1][2] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
    K[2][0] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
    K[2][1] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
    K[2][2] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
    const double det = J[0][0] * K[0][0] + J[1][0] * K[0][1] + J[2][0] * K[0][2];
    const double idet = 1.0 / det;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) K[i][j] *= idet;
    const double vol = fabs(det) / 6.0;
    // gp[a][i] = d psi_a / d x_i
    double gp[4][3];
    for (int i = 0; i < 3; ++i) {
        gp[1][i] = K[i][0]; gp[2][i] = K[i][1]; gp[3][i] = K[i][2];
        gp[0][i] = -(K[i][0] + K[i][1] + K[i][2]);
    }
    double mu[4][3], vv[4][3];
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) {
            mu[a][c] = (double)g.mu[4 * (size_t)nd[a] + c];
            vv[a][c] = (double)g.v[4 * (size_t)nd[a] + c];
        }
    double Gm[3][3], L[3][3];  // grad mu, grad v: Gm[i][j] = sum_a mu_a,i gp[a][j]
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double sm = 0.0, sv = 0.0;
            for (int a = 0; a < 4; ++a) { sm += mu[a][i] * gp[a][j]; sv += vv[a][i] * gp[a][j]; }
            Gm[i][j] = sm;
            L[i][j] = sv;
        }
    const double Gs = (double)g.G[e], Es = (double)g.E[e], As = (double)g.A[e], Bs = (double)g.B[e];
    const double v0 = (double)g.vol0[e];
    double Ji[3][3];
    for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) Ji[j][k] = (double)g.jinv[(size_t)(3 * j + k) * g.T + e];
    // F = (Ji J)^T (add_shear_elastic_stress :375-392)
    double F[3][3], FF[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += J[k][i] * Ji[j][k];
            F[i][j] = s;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += F[i][k] * F[j][k];
            FF[i][j] = s;
        }
    const double rv = v0 / vol, rr = vol / v0;
    const double E2 = Es - 2.0 * Gs / 3.0;
    const double cbulk = Gs * (1.0 - rv) + 0.5 * E2 * (rr - rv);
    double S[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S[i][j] = Gs * rv * FF[i][j] + (i == j ? cbulk - Gs : 0.0);
    // frozen noise of the step, same draws as element_kernel (add_fluctuating_stress :412-431)
    double U[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Ud[3] = {0, 0, 0}, Ub = 0.0, Uo[3] = {0, 0, 0};
    double cn = 0.0;
    if (g.calc_noise == 1) {
        uint32_t base[6], s6[6];
        for (int k = 0; k < 6; ++k) s6[k] = g.rng_state[k];
        mrg_apply(g.chunk_jump[e >> 5], s6, base);
        mrg_apply(g.lane_jump[e & 31], base, s6);
        cn = sqrt((24.0 * g.kT) / (vol * g.dt));
        Ub = mrg_rand_half(s6);
        for (int i = 0; i < 3; ++i) Ud[i] = mrg_rand_half(s6);
        for (int i = 0; i < 3; ++i) Uo[i] = mrg_rand_half(s6);
        for (int i = 0; i < 3; ++i) U[i][i] = sqrt(2.0 * As) * Ud[i] + sqrt(Bs) * Ub;
        U[0][1] = U[1][0] = sqrt(As) * Uo[0];
        U[0][2] = U[2][0] = sqrt(As) * Uo[1];
        U[1][2] = U[2][1] = sqrt(As) * Uo[2];
    }
    const double trL = L[0][0] + L[1][1] + L[2][2];
    const double trM = Gm[0][0] + Gm[1][1] + Gm[2][2];
    double T[3][3], W[3][3];
    double phi = 0.0, mFF = 0.0, mU = 0.0, mLL = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double sv = (i == j ? Bs * trL : 0.0) + As * (L[i][j] + L[j][i]);
            T[i][j] = S[i][j] + cn * U[i][j] + sv;
            W[i][j] = (i == j ? Bs * trM : 0.0) + As * (Gm[i][j] + Gm[j][i]);
            phi += Gm[i][j] * T[i][j];
            mFF += Gm[i][j] * FF[i][j];
            mU += Gm[i][j] * U[i][j];
            mLL += Gm[i][j] * (L[i][j] + L[j][i]);
        }
    // parameter gradients of -vol <grad mu, T>
    double dG = -vol * (rv * mFF + trM * (-1.0 + (1.0 - rv) - (rr - rv) / 3.0));
    double dE = -vol * 0.5 * (rr - rv) * trM;
    double dA = -vol * mLL, dB = -vol * trM * trL;
    if (g.calc_noise == 1) {
        double nA = 0.0;
        for (int i = 0; i < 3; ++i) nA += Gm[i][i] * Ud[i] / sqrt(2.0 * As);
        nA += (Gm[0][1] + Gm[1][0]) * Uo[0] / (2.0 * sqrt(As)) + (Gm[0][2] + Gm[2][0]) * Uo[1] / (2.0 * sqrt(As)) +
              (Gm[1][2] + Gm[2][1]) * Uo[2] / (2.0 * sqrt(As));
        dA += -vol * cn * nA;
        dB += -vol * cn * trM * Ub / (2.0 * sqrt(Bs));
    }
    // edge-matrix gradient: -vol [ (phi + vol Psi) K^T + (P Ji)^T - K^T Q K^T ]
    const double dcdv = Gs * v0 / (vol * vol) + 0.5 * E2 * (1.0 / v0 + v0 / (vol * vol));
    const double psi = -Gs * v0 / (vol * vol) * mFF + dcdv * trM - (cn / (2.0 * vol)) * mU;
    double P[3][3], Dm[3][3], Dv[3][3], Q[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += (Gm[i][k] + Gm[k][i]) * F[k][j];
            P[i][j] = Gs * rv * s;
            Dm[i][j] = mu[j + 1][i] - mu[0][i];
            Dv[i][j] = vv[j + 1][i] - vv[0][i];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += T[i][k] * Dm[k][j] + W[i][k] * Dv[k][j];
            Q[i][j] = s;
        }
    double KtQKt[3][3], gJ[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) s += K[k][i] * Q[k][l] * K[j][l];
            KtQKt[i][j] = s;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double pj = 0.0;  // (P Ji)^T [i][j] = (P Ji)[j][i]
            for (int k = 0; k < 3; ++k) pj += P[j][k] * Ji[k][i];
            gJ[i][j] = -vol * ((phi + vol * psi) * K[j][i] + pj - KtQKt[i][j]);
        }
    // constraint term: -sum_a w_a . (diagonal of V_e at a), w_a,i = (tau + Omega x d_a)_i v_a,i
    if (g.nmodes > 0) {
        const double *tau = g.coef, *Om = g.coef + 3;
        double w[4][3], h = 0.0, H[4][3];
        for (int a = 0; a < 4; ++a) {
            const double d[3] = {X[a][0] - g.xc[0], X[a][1] - g.xc[1], X[a][2] - g.xc[2]};
            const double z[3] = {tau[0] + (Om[1] * d[2] - Om[2] * d[1]), tau[1] + (Om[2] * d[0] - Om[0] * d[2]),
                                 tau[2] + (Om[0] * d[1] - Om[1] * d[0])};
            const double g2 = gp[a][0] * gp[a][0] + gp[a][1] * gp[a][1] + gp[a][2] * gp[a][2];
            double wsum = 0.0;
            for (int i = 0; i < 3; ++i) {
                w[a][i] = z[i] * vv[a][i];
                wsum += w[a][i];
                h += w[a][i] * ((As + Bs) * gp[a][i] * gp[a][i] + As * g2);
                dA += -vol * w[a][i] * (gp[a][i] * gp[a][i] + g2);
                dB += -vol * w[a][i] * gp[a][i] * gp[a][i];
            }
            for (int i = 0; i < 3; ++i) H[a][i] = 2.0 * w[a][i] * (As + Bs) * gp[a][i] + 2.0 * As * wsum * gp[a][i];
        }
        double HK[3][3];
        for (int i = 0; i < 3; ++i)
            for (int c = 0; c < 3; ++c) HK[i][c] = H[c + 1][i] - H[0][i];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) s += K[k][i] * HK[k][l] * K[j][l];
                gJ[i][j] += -h * vol * K[j][i] + vol * s;
            }
    }
    double *eg = g.eg + 12 * (size_t)e;
    for (int j = 0; j < 3; ++j) {
        eg[j] = -(gJ[0][j] + gJ[1][j] + gJ[2][j]);
        for (int i = 0; i < 3; ++i) eg[3 * (i + 1) + j] = gJ[i][j];
    }
    double *gt = g.gtheta + 4 * (size_t)e;
    gt[0] += dG;
    gt[1] += dE;
    gt[2] += dA;
    gt[3] += dB;
}

// lambda_n = lambda_{n+1} + sum over the node's elements of their position gradient
//            - (D_a v_a) x Omega  (the constraint's dependence on the node offsets)
template <class R>
struct AdjNodeArgs {
    int N;
    const int *inc_ptr, *inc;
    const double *eg;
    const R *v;
    const R *dinv, *diag;
    int nmodes;
    const double *coef;
    double *lam;
    const DevStatus *st;
};

template <class R>
__global__ void __launch_bounds__(256) node_vjp_kernel(AdjNodeArgs<R> g) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= g.N || g.st->abort) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int m = g.inc_ptr[a]; m < g.inc_ptr[a + 1]; ++m) {
        const int es = g.inc[m];
        const double *c = g.eg + 12 * (size_t)(es >> 2) + 3 * (es & 3);
        s[0] += c[0];
        s[1] += c[1];
        s[2] += c[2];
    }
    if (g.nmodes > 0) {
        double q[3];
        for (int c = 0; c < 3; ++c) {
            const double D = g.diag ? (double)g.diag[4 * (size_t)a + c] : 1.0 / (double)g.dinv[4 * (size_t)a + c];
            q[c] = D * (double)g.v[4 * (size_t)a + c];
        }
        const double *Om = g.coef + 3;
        s[0] -= q[1] * Om[2] - q[2] * Om[1];
        s[1] -= q[2] * Om[0] - q[0] * Om[2];
        s[2] -= q[0] * Om[1] - q[1] * Om[0];
    }
    for (int c = 0; c < 3; ++c) g.lam[4 * (size_t)a + c] += s[c];
}

}  // namespace ffea
