// kernels_batch.cuh -- many replica blobs advanced by one set of launches.
// (Included by engine_mixed.cu only: its kernels are not templates.)
//
// A batch packs B independent blobs of uneven size CSR-style: the vertex
// nodes of blob b are rows [row0_b, row0_b + nrows_b) of one global
// numbering, its elements a contiguous range, and the element, assembly,
// gather and Euler kernels of the single-blob step run unchanged over the
// concatenation (they never look across a blob's edge because no element or
// matrix block does). What is per blob is the thermal noise (one MRG32k3a
// substream per blob) and the CG: every blob has its own right-hand side,
// rigid modes, step lengths and stopping test.
//
// cg_batch_kernel is one persistent cooperative launch for the whole batch.
// The scheduler (schedule_kernel, run at the head of every step) splits the
// grid's CTAs into one group per blob, sized in proportion to the blob's
// rows x CG iterations of the previous step, so that all groups finish
// together. Each group runs the mixed-precision deflated Jacobi-PCG of
// cg_mixed_kernel on its rows with its own bounded barrier (a one-CTA group
// synchronises with __syncthreads alone) and its own partial sums, and leaves
// its loop when its own blob has converged: the per-blob convergence mask is
// the group's exit.
#pragma once

#include "batch_types.cuh"

namespace ffea {

// Rows of one blob split over the warps of its group: the group's W warps take consecutive runs of
// rppw = min(32 / tpn, ceil(nrows / W)) rows per pass, tpn lanes per row (see FFEA_ROW_LOOP).
#define BATCH_ROW_LOOP(tpn, row0, nrows, rank, gsz, a, sub, valid)                                   \
    const int sub = (threadIdx.x & 31) % (tpn);                                                      \
    const int wtot_ = (gsz) * (int)(blockDim.x >> 5);                                                \
    const int rppw_ = min(32 / (tpn), ((nrows) + wtot_ - 1) / wtot_);                                \
    const int wglob_ = (rank) * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);                    \
    const int lrow_ = (threadIdx.x & 31) / (tpn);                                                    \
    for (int a0_ = wglob_ * rppw_, la_ = a0_ + lrow_, a = (row0) + la_; a0_ < (nrows);                 \
         a0_ += wtot_ * rppw_, la_ = a0_ + lrow_, a = (row0) + la_)                                    \
        for (bool valid = lrow_ < rppw_ && la_ < (nrows), once_ = true; once_; once_ = false)

// Nodes of one blob split into equal runs, one per CTA of its group, one node per thread.
#define BATCH_NODE_LOOP(row0, nrows, rank, gsz, a)                                                    \
    for (int npb_ = ((nrows) + (gsz) - 1) / (gsz), la_ = (rank) * npb_ + (int)threadIdx.x,             \
             laend_ = min((nrows), ((rank) + 1) * npb_), a = (row0) + la_;                               \
         la_ < laend_; la_ += blockDim.x, a += blockDim.x)

__global__ void __launch_bounds__(BATCH_MAX_THREADS) cg_batch_kernel(const __grid_constant__ BatchCgArgs g) {
    __shared__ BlobCgDesc s_desc;
    __shared__ float smemf[MIXED_GATHER_NP * 32];
    __shared__ double s_sc[MIXED_GATHER_NP];
    __shared__ double s_A6[36];
    __shared__ float s_alpha, s_beta, s_tau[3], s_Om[3];
    __shared__ double s_delta;
    __shared__ int s_conv;
    DevStatus *st = g.st;
    if (st->abort) return;
    const int b = g.cta_blob[blockIdx.x];
    if (b < 0) return;
    if (threadIdx.x == 0) s_desc = g.desc[b];
    __syncthreads();
    const int row0 = s_desc.row0, nrows = s_desc.nrows, gsz = s_desc.grp_size;
    const int rank = (int)blockIdx.x - s_desc.grp_first;
    GridBarrier *gb = g.gbs + b;
    float2 *spart = g.partials + (size_t)BATCH_ROWS * s_desc.grp_first;  // set-up rows [0, 28)
    float2 *ipart = spart + (size_t)MIXED_GATHER_NP * gsz;                 // iteration rows [0, 10)
    const bool defl = s_desc.nmodes > 0;
    // set-up: node offsets d = x - x_c, moments f.f, S1_f, S2_f and M = sum Phi^T D Phi (cf. gather_mixed_kernel)
    {
        float acc[MIXED_GATHER_NP];
#pragma unroll
        for (int i = 0; i < MIXED_GATHER_NP; ++i) acc[i] = 0.f;
        BATCH_NODE_LOOP(row0, nrows, rank, gsz, a) {
            const float F0 = g.r[4 * a], F1 = g.r[4 * a + 1], F2 = g.r[4 * a + 2];
            const float dx = (float)(g.px[a] - s_desc.xc[0]), dy = (float)(g.py[a] - s_desc.xc[1]),
                        dz = (float)(g.pz[a] - s_desc.xc[2]);
            g.dpos[a] = make_float4(dx, dy, dz, 0.f);
            g.x[4 * a] = 0.f; g.x[4 * a + 1] = 0.f; g.x[4 * a + 2] = 0.f;
            acc[0] += F0 * F0 + F1 * F1 + F2 * F2;
            acc[1] += F0; acc[2] += F1; acc[3] += F2;
            acc[4] += dy * F2 - dz * F1; acc[5] += dz * F0 - dx * F2; acc[6] += dx * F1 - dy * F0;
            float phi[6][3];
            phi_cols(dx, dy, dz, phi);
            const float D[3] = {g.diag[4 * a], g.diag[4 * a + 1], g.diag[4 * a + 2]};
            int k = 7;
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = i; j < 6; ++j, ++k)
                    acc[k] += phi[i][0] * D[0] * phi[j][0] + phi[i][1] * D[1] * phi[j][1] + phi[i][2] * D[2] * phi[j][2];
        }
        df32 o[MIXED_GATHER_NP];
        block_reduce_f<MIXED_GATHER_NP>(acc, smemf, o);
        if (threadIdx.x == 0)
#pragma unroll
            for (int i = 0; i < MIXED_GATHER_NP; ++i) spart[i * gsz + rank] = make_float2(o[i].hi, o[i].lo);
    }
    bool ok = group_sync(gb, (unsigned)gsz, st, g.limit_ns);
    if (!ok) return;
    grid_sum_df<MIXED_GATHER_NP>(spart, gsz, gsz, s_sc);
    const double f2 = s_sc[0];
    mixed_setup(s_desc, s_sc, s_A6, s_tau, s_Om, &s_beta, &s_conv);
    // r = f^ (projected), z = D^{-1} r, initial r.z
    float4 *r4 = reinterpret_cast<float4 *>(g.r), *x4 = reinterpret_cast<float4 *>(g.x),
           *q4 = reinterpret_cast<float4 *>(g.q);
    const float4 *dinv4 = reinterpret_cast<const float4 *>(g.dinv), *diag4 = reinterpret_cast<const float4 *>(g.diag);
    float acc0[1] = {0.f};
    BATCH_NODE_LOOP(row0, nrows, rank, gsz, a) {
        float4 r = r4[a];
        if (defl) {
            const float4 d = g.dpos[a], D = __ldg(diag4 + a);
            r.x -= D.x * (s_tau[0] + (s_Om[1] * d.z - s_Om[2] * d.y));
            r.y -= D.y * (s_tau[1] + (s_Om[2] * d.x - s_Om[0] * d.z));
            r.z -= D.z * (s_tau[2] + (s_Om[0] * d.y - s_Om[1] * d.x));
            r4[a] = r;
        }
        const float4 di = __ldg(dinv4 + a);
        const float z0 = di.x * r.x, z1 = di.y * r.y, z2 = di.z * r.z;
        g.z[a] = make_float4(z0, z1, z2, 0.f);
        acc0[0] += r.x * z0 + r.y * z1 + r.z * z2;
    }
    const int rowz = MIXED_A_NP + MIXED_B_NP;
    {
        __syncthreads();  // smemf is reused
        df32 o[1];
        block_reduce_f<1>(acc0, smemf, o);
        if (threadIdx.x == 0) ipart[rowz * gsz + rank] = make_float2(o[0].hi, o[0].lo);
    }
    ok = group_sync(gb, (unsigned)gsz, st, g.limit_ns);
    if (ok) {
        grid_sum_df<1>(ipart + rowz * gsz, 0, gsz, s_sc);
        if (threadIdx.x == 0) s_delta = s_sc[0];
        __syncthreads();
    }
    const float4 *pold = reinterpret_cast<const float4 *>(g.pbuf0);
    float4 *pnew = reinterpret_cast<float4 *>(g.pbuf1);
    int it = 0;
    // a zero force (a blob exactly at rest without noise) has the solution x = 0: no iteration
    if (f2 == 0.0 && threadIdx.x == 0) s_conv = 1;
    for (; ok && it < g.imax && f2 != 0.0; ++it) {
        const bool first = it == 0;
        const float beta = s_beta;
        // phase A: q = V p with p = z + beta p_old formed on the fly; p.q; moments of D p
        float acc[MIXED_A_NP];
#pragma unroll
        for (int i = 0; i < MIXED_A_NP; ++i) acc[i] = 0.f;
        {
            BATCH_ROW_LOOP(g.tpn, row0, nrows, rank, gsz, a, sub, valid) {
                float q0, q1, q2;
                spmv_row_zu<3>(g, g.z, pold, beta, first, a, sub, valid, q0, q1, q2);
                if (!valid || sub != 0) continue;
                const float4 z = g.z[a];
                float p0 = z.x, p1 = z.y, p2 = z.z;
                if (!first) {
                    const float4 po = pold[a];
                    p0 = fmaf(beta, po.x, p0); p1 = fmaf(beta, po.y, p1); p2 = fmaf(beta, po.z, p2);
                }
                pnew[a] = make_float4(p0, p1, p2, 0.f);
                q4[a] = make_float4(q0, q1, q2, 0.f);
                acc[0] += p0 * q0 + p1 * q1 + p2 * q2;
                if (defl) {
                    const float4 d = g.dpos[a], D = __ldg(diag4 + a);
                    const float e0 = D.x * p0, e1 = D.y * p1, e2 = D.z * p2;
                    acc[1] += e0; acc[2] += e1; acc[3] += e2;
                    acc[4] += d.y * e2 - d.z * e1;
                    acc[5] += d.z * e0 - d.x * e2;
                    acc[6] += d.x * e1 - d.y * e0;
                }
            }
        }
        {
            df32 o[MIXED_A_NP];
            block_reduce_f<MIXED_A_NP>(acc, smemf, o);
            if (threadIdx.x == 0)
#pragma unroll
                for (int i = 0; i < MIXED_A_NP; ++i) ipart[i * gsz + rank] = make_float2(o[i].hi, o[i].lo);
        }
        if (!(ok = group_sync(gb, (unsigned)gsz, st, g.limit_ns))) break;
        grid_sum_df<MIXED_A_NP>(ipart, gsz, gsz, s_sc);
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
        const float alpha = s_alpha;
        const float t0 = s_tau[0], t1 = s_tau[1], t2 = s_tau[2], O0 = s_Om[0], O1 = s_Om[1], O2 = s_Om[2];
        // phase B: x += alpha p ; r -= alpha (q + D (tau + Omega x d)) ; r.r ; r.z
        float acc2[MIXED_B_NP] = {0.f, 0.f};
        BATCH_NODE_LOOP(row0, nrows, rank, gsz, a) {
            const float4 p = pnew[a], r = r4[a], di = __ldg(dinv4 + a);
            float4 x = x4[a], q = q4[a];
            x.x += alpha * p.x; x.y += alpha * p.y; x.z += alpha * p.z;
            x4[a] = x;
            if (defl) {
                const float4 d = g.dpos[a], D = __ldg(diag4 + a);
                q.x += D.x * (t0 + (O1 * d.z - O2 * d.y));
                q.y += D.y * (t1 + (O2 * d.x - O0 * d.z));
                q.z += D.z * (t2 + (O0 * d.y - O1 * d.x));
            }
            const float r0 = r.x - alpha * q.x, r1 = r.y - alpha * q.y, r2 = r.z - alpha * q.z;
            r4[a] = make_float4(r0, r1, r2, 0.f);
            const float z0 = di.x * r0, z1 = di.y * r1, z2 = di.z * r2;
            g.z[a] = make_float4(z0, z1, z2, 0.f);
            acc2[0] += r0 * r0 + r1 * r1 + r2 * r2;
            acc2[1] += r0 * z0 + r1 * z1 + r2 * z2;
        }
        {
            df32 o[MIXED_B_NP];
            block_reduce_f<MIXED_B_NP>(acc2, smemf, o);
            if (threadIdx.x == 0)
                for (int i = 0; i < MIXED_B_NP; ++i) ipart[(MIXED_A_NP + i) * gsz + rank] = make_float2(o[i].hi, o[i].lo);
        }
        if (!(ok = group_sync(gb, (unsigned)gsz, st, g.limit_ns))) break;
        grid_sum_df<MIXED_B_NP>(ipart + MIXED_A_NP * gsz, gsz, gsz, s_sc);
        if (threadIdx.x == 0) {
            s_conv = (f2 == 0.0 || s_sc[0] < g.eps2 * f2);
            const double delta_old = s_delta;
            s_delta = s_sc[1];
            s_beta = (float)s_delta / (float)delta_old;
        }
        __syncthreads();
        if (s_conv) {
            ++it;
            break;
        }
        const float4 *t = pold; pold = pnew; pnew = const_cast<float4 *>(t);
    }
    if (rank == 0 && threadIdx.x == 0) {
        if (!ok) {
            atomicExch(&st->abort, 1);
        } else if (!s_conv) {
            // cg_fail alone: `abort` raised now could stop a CTA of another group that has not yet
            // passed its start-up check, and its group would wait for it; batch_finish_kernel raises it
            atomicExch(&st->cg_fail, 1);
            g.blob_iters[b] = g.imax;
        } else {
            g.blob_iters[b] = it;
            atomicMax(&st->last_iters, it);
            atomicAdd(reinterpret_cast<unsigned long long *>(&st->total_iters), (unsigned long long)it);
        }
    }
}

// CTA groups for the next solve, from the rows and last iteration counts of every blob: each blob
// gets one CTA plus a share of the other C - B CTAs in proportion to rows x iterations (largest
// remainders first), so that the groups' solves take about equally long. One block.
__global__ void __launch_bounds__(1024) schedule_kernel(BlobCgDesc *desc, const int *blob_iters, int nblobs,
                                                        int ncta, int *cta_blob, const DevStatus *st) {
    __shared__ double s_wsum;
    __shared__ int s_given;
    if (st->abort) return;
    extern __shared__ double s_w[];  // nblobs weights, then nblobs remainders
    double *s_rem = s_w + nblobs;
    int *s_g = reinterpret_cast<int *>(s_rem + nblobs);
    if (threadIdx.x == 0) { s_wsum = 0.0; s_given = 0; }
    __syncthreads();
    for (int b = threadIdx.x; b < nblobs; b += blockDim.x) {
        const double w = (double)desc[b].nrows * (double)max(blob_iters[b], 1);
        s_w[b] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nblobs; ++b) s += s_w[b];  // fixed order
        s_wsum = s;
    }
    __syncthreads();
    const int spare = ncta - nblobs;
    for (int b = threadIdx.x; b < nblobs; b += blockDim.x) {
        const double share = s_wsum > 0.0 ? (double)spare * s_w[b] / s_wsum : 0.0;
        const int whole = (int)floor(share);
        s_g[b] = 1 + whole;
        s_rem[b] = share - whole;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int b = 0; b < nblobs; ++b) t += s_g[b];
        s_given = t;
    }
    __syncthreads();
    const int left = ncta - s_given;  // < nblobs: one more CTA for the `left` largest remainders
    for (int b = threadIdx.x; b < nblobs; b += blockDim.x) {
        int rankr = 0;
        const double rb = s_rem[b];
        for (int c = 0; c < nblobs; ++c) {
            const double rc = s_rem[c];
            rankr += (rc > rb || (rc == rb && c < b)) ? 1 : 0;
        }
        if (rankr < left) s_g[b] += 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int first = 0;
        for (int b = 0; b < nblobs; ++b) {
            desc[b].grp_first = first;
            desc[b].grp_size = s_g[b];
            first += s_g[b];
        }
        s_given = first;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nblobs; b += blockDim.x) {
        const int f = desc[b].grp_first, n = desc[b].grp_size;
        for (int c = f; c < f + n; ++c) cta_blob[c] = b;
    }
    for (int c = s_given + threadIdx.x; c < ncta; c += blockDim.x) cta_blob[c] = -1;
}

// closes a batch step: every blob's stream advances by its own A^(7 T_b) (when noise is on)
__global__ void batch_finish_kernel(uint32_t *rng_states, const MrgJump *step_jumps, int nblobs, DevStatus *st) {
    if (st->abort) return;
    if (st->cg_fail) {  // a blob's CG hit its cap: the step is void, later steps of the call do nothing
        if (blockIdx.x == 0 && threadIdx.x == 0) st->abort = 1;
        return;
    }
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nblobs) {
        uint32_t s[6], o[6];
        for (int k = 0; k < 6; ++k) s[k] = rng_states[6 * (size_t)b + k];
        mrg_apply(step_jumps[b], s, o);
        for (int k = 0; k < 6; ++k) rng_states[6 * (size_t)b + k] = o[k];
    }
    if (b == 0) st->steps_done += 1;
}

// every blob's strain energy (Blob::make_measurements, src/Blob.cpp:1066-1125) in FP64: one block per blob, its
// elements' energies summed in a fixed order
__global__ void __launch_bounds__(256) batch_strain_kernel(const int4 *tet, const double *px, const double *py,
                                                           const double *pz, const float *jinv, const float *G,
                                                           const float *E, const float *vol0, int T,
                                                           const int *elem_off, double *out) {
    __shared__ double smem[32];
    const int b = blockIdx.x;
    double acc[1] = {0.0};
    for (int i = elem_off[b] + threadIdx.x; i < elem_off[b + 1]; i += blockDim.x)
        acc[0] += element_strain_energy2<float>(tet[i], px, py, pz, jinv, T, i, G[i], E[i], vol0[i]);
    block_sum<1>(acc, smem);
    if (threadIdx.x == 0) out[b] = 0.5 * acc[0];
}

}  // namespace ffea
