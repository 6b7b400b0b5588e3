// batch_types.cuh -- data shared by the host and the batch kernels (kernels_batch.cuh).
#pragma once

#include "kernels_mixed.cuh"

namespace ffea {

constexpr int BATCH_MAX_THREADS = 1024;
constexpr int BATCH_ROWS = MIXED_GATHER_NP + MIXED_PARTIAL_ROWS;  // float2 partial rows per CTA

// one blob's CG description; grp_first/grp_size are rewritten by schedule_kernel every step
struct BlobCgDesc {
    int row0, nrows;
    int grp_first, grp_size;
    int nmodes, pad;
    double xc[3];
    double modes[36];
};

struct BatchCgArgs {
    static constexpr int block3 = 1;  // 3x3-block viscosity matrix (CG_nomass)
    int nblobs, tpn;
    const int *slice_ptr, *rowlen, *bcol;
    const float *val, *dinv, *diag;
    float *x, *r, *q, *pbuf0, *pbuf1;
    float4 *z;             // D^{-1} r, read by the SpMV of the blob's other rows
    float4 *dpos;
    const double *px, *py, *pz;
    const BlobCgDesc *desc;
    const int *cta_blob;   // blob of each CTA (-1: idle)
    float2 *partials;      // BATCH_ROWS per CTA; a group's block starts at BATCH_ROWS * grp_first
    GridBarrier *gbs;      // one per blob, zero at launch
    DevStatus *st;
    int *blob_iters;       // per blob: CG iterations of the last solve (imax if it failed)
    int imax;
    double eps2;
    unsigned long long limit_ns;
};

}  // namespace ffea
