// batch.cu -- host side of the replica batch: many independent blobs of
// uneven size advanced together, mixed precision, CG_nomass.
//
// The reference advances the blobs of a World one after another, each with
// the per-blob slice of World::run (src/World.cpp:1788-2059). Here B blobs
// share one packed copy of every per-node, per-element and per-matrix-slot
// array (blob b owns vertex rows [row_off[b], row_off[b+1]) and elements
// [elem_off[b], elem_off[b+1])), and one step of all of them is one CUDA
// graph: schedule, element, assembly, gather, CG, Euler and RNG kernels
// captured once and replayed. Blob b draws its thermal noise from substream b
// of the stream seeded with the package seed (RngStream::ResetNextSubstream,
// b times), in the reference's single-thread order within the blob.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"
#include "ctforces.h"
#include "ctforces_device.h"
#include "engine.h"
#include "host_model.h"
#include "mixed_elements.h"

namespace ffea {
long long launch_count();
}

using namespace ffea;
using namespace ffea::host;

struct ffea_gpu_batch {
    HostModel h;
    ffea_gpu_params p{};
    int nblobs = 0;
    std::vector<int> nall_off, row_off, elem_off, mid_off;  // nblobs + 1 each
    Arena mem;
    cudaStream_t stream = nullptr;
    int device = 0;
    double *px, *py, *pz, *vx, *vy, *vz;
    int4 *tet;
    float *jinv, *G, *E, *A, *B, *vol0, *geom;
    double *last_det;
    MixedElements me;  // FP32 node data, thread-block lists and per-block force sums of the element phase
    // Stokes noise (calc_stokes with calc_noise): per blob, 3 draws per node of its reference numbering after
    // its elements' 7 T_b, from its own stream; a midpoint's force reaches the vertices by the linearise replay
    MrgJump *sn_chunk_jump = nullptr, *sn_lane_jump = nullptr;
    int *sn_node_orig = nullptr, *sn_mid_orig = nullptr, *sn_lin_ptr = nullptr, *sn_orig_off = nullptr,
        *sn_chunk_off = nullptr;
    double *sn_mid_drag = nullptr;
    int4 *sn_lin_ev = nullptr;
    float *mid_f = nullptr;
    // constant forces (ffea_gpu_batch_load_ctforces): each blob's model, all of them on the device in the
    // concatenated numbering, and the linearise replay when only they need it
    std::vector<CtfModel> ctf_models;
    CtfDevice ctf;
    Arena lin_mem;
    int *inc_ptr, *inc, *pinned, *slice_ptr, *rowlen, *bcol, *diagk, *src_ptr, *grp_slice;
    unsigned *src;
    double *drag = nullptr;
    float *val, *dinv, *diag;
    float *x, *r, *q, *pbuf0, *pbuf1;
    float4 *zbuf = nullptr;
    float4 *dpos;
    int *elem_blob, *d_elem_off;
    uint32_t *rng_states;
    MrgJump *chunk_jump, *lane_jump, *step_jumps;
    DevStatus *st;
    GridBarrier *gbs;
    BlobCgDesc *desc;
    int *cta_blob, *blob_iters;
    float2 *partials;
    std::vector<BlobCgDesc> hdesc;
    // every blob's node state in the reference layout on the device (the blobs' n_all x 3 arrays back to
    // back), the vertex row of each vertex node and the source rows of every node (see BlobImpl)
    double *aos = nullptr;
    int *d_node_of = nullptr;
    int2 *ref_src = nullptr;
    int max_rows = 0, max_elems = 0;
    // launch configuration (ffea_gpu_batch_tune)
    int cg_threads = 256, tpn = 4, ncta = 0, ncta_cap = 0;
    // launch shapes of the force phase (ffea_gpu_batch_set_shapes): elements per block of the element kernel,
    // threads per block and slot split of the assembly (0: automatic, 1: three threads per slot, 2: one),
    // threads per block of the gather
    int asm_threads = 128, asm_split = 0, gather_threads = 256;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int kernels_per_step = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the step with event records around its CG launch (for ffea_gpu_batch_step_timed's CG time), captured on
    // first use after each capture()
    cudaGraphExec_t gexec_cg = nullptr;
    cudaEvent_t evc0 = nullptr, evc1 = nullptr;
    bool cg_events = false;  // record_step marks the CG launch

    ~ffea_gpu_batch() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (gexec_cg) cudaGraphExecDestroy(gexec_cg);
        if (evc0) cudaEventDestroy(evc0);
        if (evc1) cudaEventDestroy(evc1);
        if (graph) cudaGraphDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    int init();
    int configure(int threads, int tpn_);
    int set_shapes(int em, int at, int as, int gt);
    int time_forces(int reps, double &ms);
    int record_step();
    int capture();
    int capture_cg_timed();
    int launch_forces();
    int launch_gather();
    int launch_cg_only();
    int read_status(DevStatus &s) {
        CK(cudaMemcpyAsync(&s, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }
    int reset_flags() {
        DevStatus s{};
        int rc = read_status(s);
        if (rc) return rc;
        s.inversions = s.cg_fail = s.nonfinite = s.timeout = s.abort = 0;
        s.steps_done = 0;
        s.last_iters = 0;
        CK(cudaMemcpyAsync(st, &s, sizeof(DevStatus), cudaMemcpyHostToDevice, stream));
        return FFEA_GPU_OK;
    }
    static int status_code(const DevStatus &s) {
        if (s.timeout) return FFEA_GPU_ETIMEOUT;
        if (s.inversions) return FFEA_GPU_EINVERTED;
        if (s.cg_fail) return FFEA_GPU_ECGMAXIT;
        if (s.nonfinite) return FFEA_GPU_ENAN;
        return FFEA_GPU_OK;
    }
    int upload_desc(int only = -1) {
        const size_t b0 = only < 0 ? 0 : (size_t)only, nb = only < 0 ? hdesc.size() : 1;
        CK(cudaMemcpyAsync(desc + b0, hdesc.data() + b0, nb * sizeof(BlobCgDesc), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        return FFEA_GPU_OK;
    }
};

namespace {

// A^(2^76): the substream jump of MRG32k3a (RngStream's substreams are 2^76 draws apart)
MrgJump substream_jump() {
    Mat3 a = MRG_A1, b = MRG_A2;
    for (int i = 0; i < 76; ++i) {
        a = mat_mul(a, a, MRG_M1);
        b = mat_mul(b, b, MRG_M2);
    }
    return to_jump(a, b);
}

void apply_host(const MrgJump &J, uint32_t s[6]) {
    uint32_t o[6];
    mrg_apply(J, s, o);
    for (int k = 0; k < 6; ++k) s[k] = o[k];
}

}  // namespace

int ffea_gpu_batch::init() {
    CK(cudaGetDevice(&device));
    int major = 0, minor = 0;
    CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
    CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
    if (major != 10 || minor != 3) {
        g_last_error = "this library is built for sm_103a (GB300) only";
        return FFEA_GPU_ECUDA;
    }
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    CK(cudaEventCreate(&evc0));
    CK(cudaEventCreate(&evc1));
    const int N = h.N, T = h.T;
    for (int b = 0; b < nblobs; ++b) {
        max_rows = std::max(max_rows, row_off[b + 1] - row_off[b]);
        max_elems = std::max(max_elems, elem_off[b + 1] - elem_off[b]);
    }
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
    std::vector<float> js(9 * (size_t)T);
    for (int e = 0; e < T; ++e)
        for (int k = 0; k < 9; ++k) js[(size_t)k * T + e] = (float)h.jinv[9 * (size_t)e + k];
    CK(mem.upload(&jinv, js));
    CK(mem.upload(&G, cast_vec<float>(h.G)));
    CK(mem.upload(&E, cast_vec<float>(h.E)));
    CK(mem.upload(&A, cast_vec<float>(h.A)));
    CK(mem.upload(&B, cast_vec<float>(h.B)));
    CK(mem.upload(&vol0, cast_vec<float>(h.vol0)));
    CK(mem.upload(&last_det, h.last_det));
    CK(mem.alloc(&geom, 16 * (size_t)T));
    CK(me.init(mem, h, false, p.calc_noise == 1, elem_off));
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
    CK(mem.alloc(&val, 9 * (size_t)h.nslots));
    CK(mem.alloc(&dinv, 4 * (size_t)N));
    CK(mem.alloc(&diag, 4 * (size_t)N));
    CK(mem.alloc(&x, 4 * (size_t)N));
    CK(mem.alloc(&r, 4 * (size_t)N));
    CK(mem.alloc(&q, 4 * (size_t)N));
    CK(mem.alloc(&pbuf0, 4 * (size_t)N));
    CK(mem.alloc(&pbuf1, 4 * (size_t)N));
    CK(mem.alloc(&zbuf, (size_t)N));
    CK(mem.alloc(&dpos, (size_t)N));
    std::vector<int> eb(T);
    for (int b = 0; b < nblobs; ++b)
        for (int e = elem_off[b]; e < elem_off[b + 1]; ++e) eb[e] = b;
    CK(mem.upload(&elem_blob, eb));
    CK(mem.upload(&d_elem_off, elem_off));
    // RNG: blob b starts on substream b of the package seed's first stream
    std::vector<uint32_t> rs(6 * (size_t)nblobs);
    {
        uint32_t s[6] = {12345, 12345, 12345, 12345, 12345, 12345};
        const MrgJump sub = substream_jump();
        for (int b = 0; b < nblobs; ++b) {
            for (int k = 0; k < 6; ++k) rs[6 * (size_t)b + k] = s[k];
            apply_host(sub, s);
        }
    }
    CK(mem.upload(&rng_states, rs));
    const int nchunks = (max_elems + 31) / 32;
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
    // a step consumes 7 draws per element of the blob (noise on) and, with Stokes noise, 3 per node of its
    // reference numbering
    const bool snoise = p.calc_noise == 1 && p.calc_stokes == 1;
    std::vector<MrgJump> sj(nblobs);
    for (int b = 0; b < nblobs; ++b) {
        const uint64_t draws = p.calc_noise == 1 ? 7ull * (uint64_t)(elem_off[b + 1] - elem_off[b]) : 0ull;
        const uint64_t sdraws = snoise ? 3ull * (uint64_t)(nall_off[b + 1] - nall_off[b]) : 0ull;
        sj[b] = jump_pow(draws + sdraws);
    }
    CK(mem.upload(&step_jumps, sj));
    if (snoise) {
        // blob b's node chunk c starts A^(7 T_b + 96 c) after its stream state
        std::vector<int> choff(nblobs + 1, 0);
        std::vector<MrgJump> ncj;
        const Mat3 a96 = mat_pow(MRG_A1, 96, MRG_M1), b96 = mat_pow(MRG_A2, 96, MRG_M2);
        for (int b = 0; b < nblobs; ++b) {
            const int nch = (nall_off[b + 1] - nall_off[b] + 31) / 32;
            const uint64_t base = 7ull * (uint64_t)(elem_off[b + 1] - elem_off[b]);
            Mat3 ja = mat_pow(MRG_A1, base, MRG_M1), jb = mat_pow(MRG_A2, base, MRG_M2);
            for (int c = 0; c < nch; ++c) {
                ncj.push_back(to_jump(ja, jb));
                ja = mat_mul(a96, ja, MRG_M1);
                jb = mat_mul(b96, jb, MRG_M2);
            }
            choff[b + 1] = choff[b] + nch;
        }
        std::vector<MrgJump> nlj(32);
        for (int l = 0; l < 32; ++l) nlj[l] = jump_pow(3ull * l);
        CK(mem.upload(&sn_chunk_jump, ncj));
        CK(mem.upload(&sn_lane_jump, nlj));
        CK(mem.upload(&sn_chunk_off, choff));
        CK(mem.upload(&sn_orig_off, nall_off));
        CK(mem.upload(&sn_node_orig, h.node_of));
        CK(mem.upload(&sn_mid_orig, h.mid_nodes));
        std::vector<double> mdrag(h.mid_nodes.size());
        for (size_t m = 0; m < h.mid_nodes.size(); ++m) mdrag[m] = h.drag_all[h.mid_nodes[m]];
        CK(mem.upload(&sn_mid_drag, mdrag));
        CK(mem.upload(&sn_lin_ptr, h.lin_ptr));
        std::vector<int4> ev(h.lin_ev.size() / 4);
        for (size_t k = 0; k < ev.size(); ++k)
            ev[k] = make_int4(h.lin_ev[4 * k], h.lin_ev[4 * k + 1], h.lin_ev[4 * k + 2], -1);
        CK(mem.upload(&sn_lin_ev, ev));
        if (!h.mid_nodes.empty()) CK(mem.alloc(&mid_f, 3 * h.mid_nodes.size()));
    }
    CK(mem.alloc(&st, 1));
    CK(mem.alloc(&gbs, (size_t)nblobs));
    // CG descriptions: rows, rigid modes of each blob; an iteration estimate for the first schedule
    hdesc.assign(nblobs, BlobCgDesc{});
    std::vector<int> it0(nblobs);
    for (int b = 0; b < nblobs; ++b) {
        BlobCgDesc &d = hdesc[b];
        d.row0 = row_off[b];
        d.nrows = row_off[b + 1] - row_off[b];
        d.nmodes = rigid_modes(h, p, d.xc, d.modes, d.row0, d.nrows);
        it0[b] = std::max(10, (int)std::lround(12.0 * std::cbrt((double)d.nrows)));
    }
    CK(mem.alloc(&desc, (size_t)nblobs));
    CK(mem.upload(&blob_iters, it0));
    int rc = upload_desc();
    if (rc) return rc;
    // the grid of the largest configuration the tuner may pick bounds the per-CTA arrays
    ncta_cap = 0;
    for (int t : {128, 256, 512, 1024}) ncta_cap = std::max(ncta_cap, BatchLaunch::cg_max_grid(device, t));
    if (ncta_cap < nblobs) {
        g_last_error = "more blobs than CTAs that can be resident at once";
        return FFEA_GPU_EINPUT;
    }
    CK(mem.alloc(&cta_blob, (size_t)ncta_cap));
    CK(mem.alloc(&partials, (size_t)BATCH_ROWS * ncta_cap));
    CK(cudaDeviceSynchronize());
    // default: 256-thread CTAs (the largest size whose grid still has a CTA per blob if not), 4 lanes per row
    for (int t : {256, 128}) {
        if (BatchLaunch::cg_max_grid(device, t) >= nblobs) return configure(t, 4);
    }
    g_last_error = "no CTA size gives one CTA per blob";
    return FFEA_GPU_EINPUT;
}

// pick the CG CTA size and lanes per matrix row, and capture the step graph for them
int ffea_gpu_batch::configure(int threads, int tpn_) {
    const int grid = BatchLaunch::cg_max_grid(device, threads);
    if (grid < nblobs || grid > ncta_cap || !(tpn_ == 1 || tpn_ == 2 || tpn_ == 4 || tpn_ == 8)) {
        g_last_error = "invalid batch launch configuration";
        return FFEA_GPU_EINPUT;
    }
    cg_threads = threads;
    tpn = tpn_;
    ncta = grid;
    return capture();
}

// the force phase's launch shapes; the step graph is captured again
int ffea_gpu_batch::set_shapes(int em, int at, int as, int gt) {
    auto ok = [](int t) { return t == 64 || t == 128 || t == 256; };
    if (!ok(em) || !ok(at) || !ok(gt) || as < 0 || as > 2) {
        g_last_error = "invalid batch launch shapes";
        return FFEA_GPU_EINPUT;
    }
    if (em != me.threads) {
        CK(cudaStreamSynchronize(stream));
        CK(me.set_threads(h, em));
    }
    asm_threads = at;
    asm_split = as;
    gather_threads = gt;
    return capture();
}

// mean time of the force phase (node preparation, elements, assembly, node forces) over `reps` launches
// after one warm-up, at the current positions; changes no state the step reads
int ffea_gpu_batch::time_forces(int reps, double &ms) {
    double tot = 0.0;
    for (int k = 0; k <= reps; ++k) {
        CK(cudaEventRecord(ev0, stream));
        int rc = launch_forces();
        if (!rc) rc = launch_gather();
        if (rc) return rc;
        CK(cudaEventRecord(ev1, stream));
        CK(cudaEventSynchronize(ev1));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, ev0, ev1));
        if (k > 0) tot += t;
    }
    ms = tot / reps;
    return FFEA_GPU_OK;
}

// one step of every blob, as launched into `stream` (captured by capture())
int ffea_gpu_batch::record_step() {
    CK(BatchLaunch::schedule(desc, blob_iters, nblobs, ncta, cta_blob, st, stream));
    int rc = launch_forces();
    if (!rc) rc = launch_gather();
    if (rc) return rc;
    if (cg_events) CK(cudaEventRecordWithFlags(evc0, stream, cudaEventRecordExternal));
    rc = launch_cg_only();
    if (rc) return rc;
    if (cg_events) CK(cudaEventRecordWithFlags(evc1, stream, cudaEventRecordExternal));
    EulerArgs<float> eu{};
    eu.N = h.N; eu.nomass = 1; eu.dt = p.dt; eu.x = x;
    eu.px = px; eu.py = py; eu.pz = pz; eu.vx = vx; eu.vy = vy; eu.vz = vz;
    eu.st = st;
    CK(Launch<float>::euler(eu, stream));
    CK(BatchLaunch::finish(rng_states, step_jumps, nblobs, st, stream));
    return FFEA_GPU_OK;
}

// element stress and forces, then the viscosity matrices assembled into the packed SELL matrix
int ffea_gpu_batch::launch_forces() {
    ElemArgs<float> ea{};
    ea.T = h.T;
    ea.nomass = 1;
    ea.calc_noise = p.calc_noise;
    ea.kT = (float)p.kT;
    ea.dt = (float)p.dt;
    ea.tet = tet;
    ea.px = px; ea.py = py; ea.pz = pz;
    ea.vx = vx; ea.vy = vy; ea.vz = vz;
    ea.jinv = jinv;
    ea.G = G; ea.E = E; ea.A = A; ea.B = B; ea.vol0 = vol0;
    ea.last_det = last_det;
    ea.geom = geom;
    ea.rng_state = rng_states;
    ea.elem_blob = elem_blob;
    ea.elem_off = d_elem_off;
    ea.chunk_jump = chunk_jump;
    ea.lane_jump = lane_jump;
    ea.st = st;
    me.fill(ea);
    CK(me.prep(px, py, pz, vx, vy, vz, rng_states, chunk_jump, stream));
    CK(MixedLaunch::element(ea, true, stream));
    AsmArgs<float> aa{};
    aa.N = h.N;
    aa.nslots = h.nslots; aa.grp_slice = grp_slice;
    aa.slice_ptr = slice_ptr; aa.rowlen = rowlen; aa.bcol = bcol; aa.diagk = diagk;
    aa.src_ptr = src_ptr; aa.src = src;
    aa.geom = geom; aa.A = A; aa.B = B;
    aa.drag = (p.calc_stokes == 1) ? drag : nullptr;
    aa.val = val; aa.dinv = dinv; aa.diag = diag; aa.st = st;
    aa.threads = asm_threads;
    aa.split = asm_split;
    CK(Launch<float>::assemble(aa, stream));
    return FFEA_GPU_OK;
}

// node forces gathered from the elements: f, and r = f for the CG
int ffea_gpu_batch::launch_gather() {
    GatherArgs<float> ga{};
    ga.N = h.N;
    ga.mode = 2;
    ga.inc_ptr = inc_ptr; ga.inc = inc; ga.ef = nullptr; ga.pinned = pinned;
    ga.parts = me.parts; ga.part_ptr = me.part_ptr;
    ga.drag = nullptr;
    ga.vx = vx; ga.vy = vy; ga.vz = vz;
    ga.dinv = dinv; ga.x = x; ga.r = r;  // no FP64 copy of the force: the batch CG starts from r
    ga.partials = nullptr; ga.stride = 0; ga.st = st; ga.gb = nullptr;
    ga.dpos = dpos; ga.px = px; ga.py = py; ga.pz = pz; ga.diag = diag;
    NodeForces &sn = ga.sn;
    ctf.fill(sn);
    sn.lin_ptr = sn_lin_ptr;
    sn.lin_ev = sn_lin_ev;
    if (sn_chunk_jump) {
        sn.noise = 1;
        sn.kT = p.kT;
        sn.dt = p.dt;
        sn.rng_state = rng_states;
        sn.chunk_jump = sn_chunk_jump;
        sn.lane_jump = sn_lane_jump;
        sn.node_orig = sn_node_orig;
        sn.node_drag = drag;
        sn.mid_orig = sn_mid_orig;
        sn.mid_drag = sn_mid_drag;
        sn.orig_off = sn_orig_off;
        sn.chunk_off = sn_chunk_off;
        sn.nblobs = nblobs;
    }
    sn.on = sn.noise || sn.lin_ptr != nullptr;
    CK(ctf.launch(stream));
    // each midpoint's force once per step (the vertices' linearise replay reads it up to ~20 times)
    if (sn.lin_ptr && mid_f && (sn.noise || ctf.mid || ctf.mface_ptr)) {
        CK(Launch<float>::mid_force(sn, (int)h.mid_nodes.size(), mid_f, st, stream));
        sn.mid_f = mid_f;
    }
    ga.threads = gather_threads;
    CK(Launch<float>::gather(ga, (h.N + gather_threads - 1) / gather_threads, stream));
    return FFEA_GPU_OK;
}

// barrier reset + the persistent CG over every blob
int ffea_gpu_batch::launch_cg_only() {
    CK(cudaMemsetAsync(gbs, 0, (size_t)nblobs * sizeof(GridBarrier), stream));
    BatchCgArgs ca{};
    ca.nblobs = nblobs;
    ca.tpn = tpn;
    ca.slice_ptr = slice_ptr; ca.rowlen = rowlen; ca.bcol = bcol;
    ca.val = val; ca.dinv = dinv; ca.diag = diag;
    ca.x = x; ca.r = r; ca.q = q; ca.pbuf0 = pbuf0; ca.pbuf1 = pbuf1; ca.z = zbuf;
    ca.dpos = dpos;
    ca.px = px; ca.py = py; ca.pz = pz;
    ca.desc = desc;
    ca.cta_blob = cta_blob;
    ca.partials = partials;
    ca.gbs = gbs;
    ca.st = st;
    ca.blob_iters = blob_iters;
    ca.imax = p.max_iterations_cg;
    ca.eps2 = p.epsilon2;
    ca.limit_ns = 2000000000ull;
    CK(BatchLaunch::cg(ca, ncta, cg_threads, stream));
    return FFEA_GPU_OK;
}

int ffea_gpu_batch::capture() {
    if (gexec_cg) { cudaGraphExecDestroy(gexec_cg); gexec_cg = nullptr; }
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    const long long l0 = launch_count();
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = record_step();
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    graph = g;
    kernels_per_step = (int)(launch_count() - l0);
    count_launch(-kernels_per_step);  // counted again on every replay
    CK(cudaGraphInstantiate(&gexec, graph, 0));
    return FFEA_GPU_OK;
}

// the same step with event record nodes around its CG launch
int ffea_gpu_batch::capture_cg_timed() {
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const long long l0 = launch_count();
    cg_events = true;
    const int rc = record_step();
    cg_events = false;
    count_launch((int)(l0 - launch_count()));
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : cuda_fail(e, "cudaStreamEndCapture");
    }
    const cudaError_t ei = cudaGraphInstantiate(&gexec_cg, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        gexec_cg = nullptr;
        return cuda_fail(ei, "cudaGraphInstantiate");
    }
    return FFEA_GPU_OK;
}

namespace {

int check_batch_params(const ffea_gpu_params *p) {
    if (!p || !(p->dt > 0) || p->max_iterations_cg < 0) {
        g_last_error = "invalid parameters";
        return FFEA_GPU_EINPUT;
    }
    if (p->solver != FFEA_GPU_NOMASS_CG || p->precision != FFEA_GPU_MIXED) {
        g_last_error = "a batch runs the CG_nomass solver in mixed precision";
        return FFEA_GPU_EINPUT;
    }
    return FFEA_GPU_OK;
}

}  // namespace

extern "C" {

int ffea_gpu_batch_create(const ffea_gpu_mesh *meshes, int nblobs, const ffea_gpu_params *params,
                          ffea_gpu_batch **out) {
    if (!out || !meshes || nblobs <= 0) return FFEA_GPU_EINPUT;
    if (nblobs > FFEA_GPU_BATCH_MAX_BLOBS) {
        g_last_error = "too many blobs in one batch";
        return FFEA_GPU_EINPUT;
    }
    *out = nullptr;
    int rc = check_batch_params(params);
    if (rc) return rc;
    ffea_gpu_batch *bt = nullptr;
    try {
        bt = new ffea_gpu_batch();
        bt->p = *params;
        bt->nblobs = nblobs;
        // one combined structure: blob b's nodes, elements and pins follow blob b-1's
        long long nall = 0, T = 0, npin = 0;
        for (int b = 0; b < nblobs; ++b) {
            const ffea_gpu_mesh &m = meshes[b];
            if (m.num_nodes <= 0 || m.num_elements <= 0 || m.num_pinned < 0 || !m.pos || !m.tets || !m.rho ||
                !m.A || !m.B || !m.G || !m.E || (m.num_pinned > 0 && !m.pinned) ||
                (params->calc_stokes == 1 && !m.stokes_radius)) {
                g_last_error = "blob " + std::to_string(b) + ": empty mesh or missing arrays";
                delete bt;
                return FFEA_GPU_EINPUT;
            }
            nall += m.num_nodes;
            T += m.num_elements;
            npin += m.num_pinned;
        }
        if (nall >= (1ll << 31) || T >= (1ll << 28)) {
            g_last_error = "batch too large for 32-bit node or 28-bit element indices";
            delete bt;
            return FFEA_GPU_EINPUT;
        }
        std::vector<double> pos(3 * nall), rho(T), A(T), B(T), G(T), E(T), sr(nall, 0.0);
        std::vector<int> tets(10 * T), pins;
        pins.reserve(npin);
        bt->nall_off.assign(nblobs + 1, 0);
        bt->elem_off.assign(nblobs + 1, 0);
        for (int b = 0; b < nblobs; ++b) {
            const ffea_gpu_mesh &m = meshes[b];
            const int n0 = bt->nall_off[b], e0 = bt->elem_off[b];
            std::copy(m.pos, m.pos + 3 * (size_t)m.num_nodes, pos.begin() + 3 * (size_t)n0);
            if (m.stokes_radius) std::copy(m.stokes_radius, m.stokes_radius + m.num_nodes, sr.begin() + n0);
            for (size_t k = 0; k < 10 * (size_t)m.num_elements; ++k) {
                const int x = m.tets[k];
                if (x < 0 || x >= m.num_nodes) {
                    g_last_error = "blob " + std::to_string(b) + ": element references an out of bounds node";
                    delete bt;
                    return FFEA_GPU_EINPUT;
                }
                tets[10 * (size_t)e0 + k] = x + n0;
            }
            std::copy(m.rho, m.rho + m.num_elements, rho.begin() + e0);
            std::copy(m.A, m.A + m.num_elements, A.begin() + e0);
            std::copy(m.B, m.B + m.num_elements, B.begin() + e0);
            std::copy(m.G, m.G + m.num_elements, G.begin() + e0);
            std::copy(m.E, m.E + m.num_elements, E.begin() + e0);
            for (int k = 0; k < m.num_pinned; ++k) {
                if (m.pinned[k] < 0 || m.pinned[k] >= m.num_nodes) {
                    g_last_error = "blob " + std::to_string(b) + ": pinned node index out of bounds";
                    delete bt;
                    return FFEA_GPU_EINPUT;
                }
                pins.push_back(m.pinned[k] + n0);
            }
            bt->nall_off[b + 1] = n0 + m.num_nodes;
            bt->elem_off[b + 1] = e0 + m.num_elements;
        }
        ffea_gpu_mesh all{(int)nall, (int)T, (int)pins.size(), pos.data(), tets.data(), rho.data(), A.data(),
                          B.data(), G.data(), E.data(), sr.data(), pins.empty() ? nullptr : pins.data()};
        rc = build_model(&all, params, bt->h);
        if (rc) {
            delete bt;
            return rc;
        }
        // vertex rows and midpoints per blob (the compaction keeps the node order, so they are contiguous)
        const HostModel &h = bt->h;
        bt->row_off.assign(nblobs + 1, 0);
        bt->mid_off.assign(nblobs + 1, 0);
        for (int b = 0, k = 0, m = 0; b < nblobs; ++b) {
            while (k < h.N && h.node_of[k] < bt->nall_off[b + 1]) ++k;
            while (m < (int)h.mid_nodes.size() && h.mid_nodes[m] < bt->nall_off[b + 1]) ++m;
            bt->row_off[b + 1] = k;
            bt->mid_off[b + 1] = m;
        }
        for (int b = 0; b < nblobs; ++b)
            if (bt->row_off[b + 1] == bt->row_off[b]) {
                g_last_error = "blob " + std::to_string(b) + " has no vertex nodes";
                delete bt;
                return FFEA_GPU_EINPUT;
            }
    } catch (std::bad_alloc &) {
        delete bt;
        return FFEA_GPU_ENOMEM;
    }
    rc = bt->init();
    if (rc) {
        delete bt;
        return rc;
    }
    *out = bt;
    return FFEA_GPU_OK;
}

void ffea_gpu_batch_destroy(ffea_gpu_batch *bt) { delete bt; }

int ffea_gpu_batch_sizes(ffea_gpu_batch *bt, int *nblobs, int *nodes, int *elements, long long *blocks) {
    if (!bt) return FFEA_GPU_EINPUT;
    if (nblobs) *nblobs = bt->nblobs;
    if (nodes) *nodes = bt->h.N;
    if (elements) *elements = bt->h.T;
    if (blocks) {
        long long s = 0;
        for (int a = 0; a < bt->h.N; ++a) s += bt->h.rowlen[a];
        *blocks = s;
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_blob_sizes(ffea_gpu_batch *bt, int blob, int *num_nodes, int *vertex_nodes, int *elements) {
    if (!bt || blob < 0 || blob >= bt->nblobs) return FFEA_GPU_EINPUT;
    if (num_nodes) *num_nodes = bt->nall_off[blob + 1] - bt->nall_off[blob];
    if (vertex_nodes) *vertex_nodes = bt->row_off[blob + 1] - bt->row_off[blob];
    if (elements) *elements = bt->elem_off[blob + 1] - bt->elem_off[blob];
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_step(ffea_gpu_batch *bt, int nsteps, int *steps_done) {
    if (!bt || nsteps < 0) return FFEA_GPU_EINPUT;
    int rc = bt->reset_flags();
    if (rc) return rc;
    for (int i = 0; i < nsteps; ++i) {
        CK(cudaGraphLaunch(bt->gexec, bt->stream));
        count_launch(bt->kernels_per_step);
    }
    DevStatus s{};
    rc = bt->read_status(s);
    if (rc) return rc;
    if (steps_done) *steps_done = s.steps_done;
    return ffea_gpu_batch::status_code(s);
}

int ffea_gpu_batch_step_timed(ffea_gpu_batch *bt, int nsteps, long long flush_bytes, int *steps_done,
                              double *step_ms, double *cg_ms) {
    if (!bt || nsteps < 0 || flush_bytes < 0) return FFEA_GPU_EINPUT;
    int rc = bt->reset_flags();
    if (rc) return rc;
    if (cg_ms && !bt->gexec_cg && (rc = bt->capture_cg_timed())) return rc;
    cudaGraphExec_t ge = cg_ms ? bt->gexec_cg : bt->gexec;
    double tcg = 0.0;
    void *scratch = nullptr;
    if (flush_bytes > 0) CK(cudaMalloc(&scratch, (size_t)flush_bytes));
    double tot = 0.0;
    for (int i = 0; i < nsteps && rc == FFEA_GPU_OK; ++i) {
        cudaError_t e = cudaSuccess;
        if (scratch) e = cudaMemsetAsync(scratch, i & 0xff, (size_t)flush_bytes, bt->stream);
        if (e == cudaSuccess) e = cudaEventRecord(bt->ev0, bt->stream);
        if (e == cudaSuccess) e = cudaGraphLaunch(ge, bt->stream);
        if (e == cudaSuccess) e = cudaEventRecord(bt->ev1, bt->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(bt->ev1);
        float ms = 0.f, mc = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, bt->ev0, bt->ev1);
        if (e == cudaSuccess && cg_ms) e = cudaEventElapsedTime(&mc, bt->evc0, bt->evc1);
        tcg += mc;
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "timed batch step");
            break;
        }
        count_launch(bt->kernels_per_step);
        tot += ms;
    }
    if (scratch) cudaFree(scratch);
    if (rc) return rc;
    DevStatus s{};
    rc = bt->read_status(s);
    if (rc) return rc;
    if (steps_done) *steps_done = s.steps_done;
    if (step_ms) *step_ms = tot;
    if (cg_ms) *cg_ms = tcg;
    return ffea_gpu_batch::status_code(s);
}

// blobs [b0, b1) in the reference layout: assembled on the device, one copy out
static int batch_get_range(ffea_gpu_batch *bt, int b0, int b1, double *pos, double *vel) {
    const int n0 = bt->nall_off[b0], n = bt->nall_off[b1] - n0;
    auto fill = [&](double *out, const double *dx, const double *dy, const double *dz, bool mids) -> int {
        CK(launch_aos_gather(dx, dy, dz, bt->ref_src + n0, n, mids ? 1 : 0, bt->aos + 3 * (size_t)n0, bt->stream));
        CK(cudaMemcpyAsync(out, bt->aos + 3 * (size_t)n0, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                           bt->stream));
        CK(cudaStreamSynchronize(bt->stream));
        return FFEA_GPU_OK;
    };
    int rc;
    if (pos && (rc = fill(pos, bt->px, bt->py, bt->pz, true))) return rc;
    if (vel && (rc = fill(vel, bt->vx, bt->vy, bt->vz, false))) return rc;
    return FFEA_GPU_OK;
}

// blobs [b0, b1) from the reference layout: one copy in, the vertex rows picked out on the device; then the
// host's copy of the positions and the blobs' rigid modes
static int batch_set_range(ffea_gpu_batch *bt, int b0, int b1, const double *pos, const double *vel) {
    HostModel &h = bt->h;
    const int n0 = bt->nall_off[b0], n = bt->nall_off[b1] - n0;
    const int r0 = bt->row_off[b0], nr = bt->row_off[b1] - r0;
    auto put = [&](const double *in, double *dx, double *dy, double *dz) -> int {
        CK(cudaMemcpyAsync(bt->aos + 3 * (size_t)n0, in, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                           bt->stream));
        CK(launch_aos_scatter(bt->aos, bt->d_node_of + r0, nr, dx + r0, dy + r0, dz + r0, bt->stream));
        return FFEA_GPU_OK;
    };
    int rc;
    if (vel && (rc = put(vel, bt->vx, bt->vy, bt->vz))) return rc;
    if (pos && (rc = put(pos, bt->px, bt->py, bt->pz))) return rc;
    if (!pos) {
        CK(cudaStreamSynchronize(bt->stream));  // the caller may reuse its arrays on return
        return FFEA_GPU_OK;
    }
    // while the positions travel: each blob's centroid in one pass over its vertex rows; the host copy of the
    // positions is kept for the pinned rows only (all the rigid modes need)
    for (int b = b0; b < b1; ++b) {
        BlobCgDesc &d = bt->hdesc[b];
        double sum[3] = {0.0, 0.0, 0.0};
        for (int k = d.row0; k < d.row0 + d.nrows; ++k) {
            const double *q = pos + 3 * (size_t)(h.node_of[k] - n0);
            sum[0] += q[0]; sum[1] += q[1]; sum[2] += q[2];
            if (h.pinned[k])
                for (int c = 0; c < 3; ++c) h.pos[3 * (size_t)k + c] = q[c];
        }
        for (int c = 0; c < 3; ++c) d.xc[c] = sum[c] / std::max(d.nrows, 1);
        d.nmodes = rigid_modes_about(h, bt->p, d.xc, d.modes, d.row0, d.nrows);
    }
    return bt->upload_desc(b1 - b0 == 1 ? b0 : -1);  // ends with a stream synchronisation
}

int ffea_gpu_batch_get_state(ffea_gpu_batch *bt, int blob, double *pos, double *vel) {
    if (!bt || blob < 0 || blob >= bt->nblobs) return FFEA_GPU_EINPUT;
    return batch_get_range(bt, blob, blob + 1, pos, vel);
}

int ffea_gpu_batch_set_state(ffea_gpu_batch *bt, int blob, const double *pos, const double *vel) {
    if (!bt || blob < 0 || blob >= bt->nblobs) return FFEA_GPU_EINPUT;
    return batch_set_range(bt, blob, blob + 1, pos, vel);
}

int ffea_gpu_batch_get_states(ffea_gpu_batch *bt, double *pos, double *vel) {
    if (!bt) return FFEA_GPU_EINPUT;
    return batch_get_range(bt, 0, bt->nblobs, pos, vel);
}

int ffea_gpu_batch_set_states(ffea_gpu_batch *bt, const double *pos, const double *vel) {
    if (!bt) return FFEA_GPU_EINPUT;
    return batch_set_range(bt, 0, bt->nblobs, pos, vel);
}

int ffea_gpu_batch_set_rng_state(ffea_gpu_batch *bt, int blob, const uint32_t s[6]) {
    if (!bt || blob < 0 || blob >= bt->nblobs || !s || !valid_seed(s)) return FFEA_GPU_EINPUT;
    CK(cudaMemcpyAsync(bt->rng_states + 6 * (size_t)blob, s, 6 * sizeof(uint32_t), cudaMemcpyHostToDevice,
                       bt->stream));
    CK(cudaStreamSynchronize(bt->stream));
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_load_ctforces(ffea_gpu_batch *bt, int blob, const char *ctf_file, const char *surf_file,
                                 int blob_index) {
    if (!bt || blob < 0 || blob >= bt->nblobs || !ctf_file) return FFEA_GPU_EINPUT;
    const int nb = bt->nblobs;
    CtfModel cm;
    std::string err;
    int rc = load_ctforces(ctf_file, surf_file, blob_index, bt->nall_off[blob + 1] - bt->nall_off[blob], cm, err);
    if (rc) {
        g_last_error = err;
        return rc;
    }
    if ((int)bt->ctf_models.size() != nb) {
        bt->ctf_models.resize(nb);
        for (int b = 0; b < nb; ++b) empty_ctforces(bt->nall_off[b + 1] - bt->nall_off[b], bt->ctf_models[b]);
    }
    std::swap(bt->ctf_models[blob], cm);  // cm now holds the blob's previous forces
    CtfModel all;
    concat_ctforces(bt->ctf_models, bt->nall_off, all);
    CK(cudaStreamSynchronize(bt->stream));
    const cudaError_t be = bt->ctf.build(bt->h, all, bt->px, bt->py, bt->pz, bt->st);
    if (be != cudaSuccess) {
        // keep the batch consistent: the previous forces back on the device, the step graph re-captured
        std::swap(bt->ctf_models[blob], cm);
        concat_ctforces(bt->ctf_models, bt->nall_off, all);
        bt->ctf.build(bt->h, all, bt->px, bt->py, bt->pz, bt->st);
        bt->capture();
        return cuda_fail(be, "batch_load_ctforces");
    }
    const int M = (int)bt->h.mid_nodes.size();
    if (bt->ctf.mid_force && !bt->mid_f && M > 0) CK(bt->mem.alloc(&bt->mid_f, 3 * (size_t)M));
    // midpoints that carry force need the linearisation replay (already there with Stokes noise)
    if (bt->ctf.mid_force && !bt->sn_lin_ptr) {
        build_linearise_events(bt->h);
        CK(bt->lin_mem.upload(&bt->sn_lin_ptr, bt->h.lin_ptr));
        std::vector<int4> ev(bt->h.lin_ev.size() / 4);
        for (size_t k = 0; k < ev.size(); ++k)
            ev[k] = make_int4(bt->h.lin_ev[4 * k], bt->h.lin_ev[4 * k + 1], bt->h.lin_ev[4 * k + 2], -1);
        CK(bt->lin_mem.upload(&bt->sn_lin_ev, ev));
    }
    return bt->capture();
}

int ffea_gpu_batch_strain_energies(ffea_gpu_batch *bt, double *out) {
    if (!bt || !out) return FFEA_GPU_EINPUT;
    double *d = nullptr;
    CK(cudaMallocAsync(&d, sizeof(double) * bt->nblobs, bt->stream));
    cudaError_t e = BatchLaunch::strain(bt->tet, bt->px, bt->py, bt->pz, bt->jinv, bt->G, bt->E, bt->vol0, bt->h.T,
                                        bt->d_elem_off, bt->nblobs, d, bt->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d, sizeof(double) * bt->nblobs, cudaMemcpyDeviceToHost, bt->stream);
    cudaFreeAsync(d, bt->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(bt->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch_strain_energies");
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_get_rng_state(ffea_gpu_batch *bt, int blob, uint32_t s[6]) {
    if (!bt || blob < 0 || blob >= bt->nblobs || !s) return FFEA_GPU_EINPUT;
    CK(cudaMemcpyAsync(s, bt->rng_states + 6 * (size_t)blob, 6 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       bt->stream));
    CK(cudaStreamSynchronize(bt->stream));
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_cg_iterations(ffea_gpu_batch *bt, int *last_per_blob, long long *total) {
    if (!bt) return FFEA_GPU_EINPUT;
    if (last_per_blob)
        CK(cudaMemcpyAsync(last_per_blob, bt->blob_iters, bt->nblobs * sizeof(int), cudaMemcpyDeviceToHost,
                           bt->stream));
    DevStatus s{};
    int rc = bt->read_status(s);
    if (rc) return rc;
    if (total) *total = s.total_iters;
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_config(ffea_gpu_batch *bt, int *cg_threads, int *threads_per_row, int *ctas) {
    if (!bt) return FFEA_GPU_EINPUT;
    if (cg_threads) *cg_threads = bt->cg_threads;
    if (threads_per_row) *threads_per_row = bt->tpn;
    if (ctas) *ctas = bt->ncta;
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_shapes(ffea_gpu_batch *bt, int *element_threads, int *assembly_threads, int *assembly_split,
                          int *gather_threads) {
    if (!bt) return FFEA_GPU_EINPUT;
    if (element_threads) *element_threads = bt->me.threads;
    if (assembly_threads) *assembly_threads = bt->asm_threads;
    if (assembly_split) *assembly_split = bt->asm_split;
    if (gather_threads) *gather_threads = bt->gather_threads;
    return FFEA_GPU_OK;
}

int ffea_gpu_batch_set_shapes(ffea_gpu_batch *bt, int element_threads, int assembly_threads, int assembly_split,
                              int gather_threads) {
    if (!bt) return FFEA_GPU_EINPUT;
    return bt->set_shapes(element_threads, assembly_threads, assembly_split, gather_threads);
}

int ffea_gpu_batch_set_config(ffea_gpu_batch *bt, int cg_threads, int threads_per_row) {
    if (!bt) return FFEA_GPU_EINPUT;
    return bt->configure(cg_threads, threads_per_row);
}

int ffea_gpu_batch_tune(ffea_gpu_batch *bt, int solves, double *best_ms) {
    if (!bt || solves <= 0) return FFEA_GPU_EINPUT;
    int rc = bt->reset_flags();
    if (rc) return rc;
    DevStatus s0{};
    if ((rc = bt->read_status(s0))) return rc;
    // the force phase's launch shapes, one at a time (coordinate search): elements per block, then the
    // assembly's threads per block and slot split, then the gather's threads per block
    const int keep_threads = bt->cg_threads, keep_tpn = bt->tpn;
    const int keep_em = bt->me.threads, keep_at = bt->asm_threads, keep_as = bt->asm_split,
              keep_gt = bt->gather_threads;
    auto restore = [&]() {
        if (bt->me.threads != keep_em) {
            cudaStreamSynchronize(bt->stream);
            bt->me.set_threads(bt->h, keep_em);
        }
        bt->asm_threads = keep_at;
        bt->asm_split = keep_as;
        bt->gather_threads = keep_gt;
    };
    {
        double ms = 0.0, fbest = 1e300;
        int b_em = keep_em;
        for (int em : {64, 128, 256}) {
            if (em != bt->me.threads) {
                CK(cudaStreamSynchronize(bt->stream));
                CK(bt->me.set_threads(bt->h, em));
            }
            if ((rc = bt->time_forces(solves, ms))) break;
            if (ms < fbest) { fbest = ms; b_em = em; }
        }
        if (!rc && b_em != bt->me.threads) {
            CK(cudaStreamSynchronize(bt->stream));
            CK(bt->me.set_threads(bt->h, b_em));
        }
        int b_at = keep_at, b_as = keep_as;
        fbest = 1e300;
        for (int at : {64, 128, 256}) {
            for (int as : {1, 2}) {
                if (rc) break;
                bt->asm_threads = at;
                bt->asm_split = as;
                if ((rc = bt->time_forces(solves, ms))) break;
                if (ms < fbest) { fbest = ms; b_at = at; b_as = as; }
            }
        }
        bt->asm_threads = b_at;
        bt->asm_split = b_as;
        int b_gt = keep_gt;
        fbest = 1e300;
        for (int gt : {64, 128, 256}) {
            if (rc) break;
            bt->gather_threads = gt;
            if ((rc = bt->time_forces(solves, ms))) break;
            if (ms < fbest) { fbest = ms; b_gt = gt; }
        }
        bt->gather_threads = b_gt;
        DevStatus s{};
        if (!rc) rc = bt->read_status(s);
        if (!rc) rc = ffea_gpu_batch::status_code(s);
        if (rc) {
            restore();
            bt->configure(keep_threads, keep_tpn);
            return rc;
        }
    }
    // forces and matrix of the current positions; no position or RNG update
    if ((rc = bt->launch_forces())) return rc;
    auto prepare = [&]() -> int {
        int r2 = bt->launch_gather();
        if (r2) return r2;
        CK(BatchLaunch::schedule(bt->desc, bt->blob_iters, bt->nblobs, bt->ncta, bt->cta_blob, bt->st, bt->stream));
        return FFEA_GPU_OK;
    };
    int best_t = keep_threads, best_p = keep_tpn;
    double best = 1e300;
    for (int t : {128, 256, 512, 1024}) {
        const int grid = BatchLaunch::cg_max_grid(bt->device, t);
        if (grid < bt->nblobs || grid > bt->ncta_cap) continue;
        for (int p : {1, 2, 4, 8}) {
            bt->cg_threads = t;
            bt->tpn = p;
            bt->ncta = grid;
            double tot = 0.0;
            for (int k = 0; k <= solves && rc == FFEA_GPU_OK; ++k) {
                if ((rc = prepare())) break;
                cudaError_t e = cudaEventRecord(bt->ev0, bt->stream);
                if (e == cudaSuccess) rc = bt->launch_cg_only();
                if (rc) break;
                if (e == cudaSuccess) e = cudaEventRecord(bt->ev1, bt->stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(bt->ev1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, bt->ev0, bt->ev1);
                if (e != cudaSuccess) rc = cuda_fail(e, "batch tune");
                if (k > 0) tot += ms;  // the first solve of each configuration is a warm-up
            }
            if (rc) break;
            DevStatus s{};
            if ((rc = bt->read_status(s))) break;
            if ((rc = ffea_gpu_batch::status_code(s))) break;
            if (tot / solves < best) {
                best = tot / solves;
                best_t = t;
                best_p = p;
            }
        }
        if (rc) break;
    }
    // the tuning solves are not steps: put the status counters back
    if (!rc) {
        CK(cudaMemcpyAsync(bt->st, &s0, sizeof(DevStatus), cudaMemcpyHostToDevice, bt->stream));
        CK(cudaStreamSynchronize(bt->stream));
    }
    if (rc) {
        restore();
        bt->configure(keep_threads, keep_tpn);
        return rc;
    }
    if (best_ms) *best_ms = best;
    return bt->configure(best_t, best_p);
}

}  // extern "C"
