// host_model.h -- host-side model of a blob, shared by the single-blob and batch engines.
//
// HostModel is what the reference's Blob holds after Blob::init, reduced to
// the vertex ("linear") nodes: rest state (calc_rest_state_info,
// src/Blob.cpp:3080-3143), node-element incidence
// (calculate_node_element_connectivity, src/Blob.cpp:3284-3314), the fixed
// 3x3-block sparsity pattern with its per-slot assembly sources
// (NoMassCGSolver::init, src/NoMassCGSolver.cpp:56-153), and the mass data of
// the two inertial solvers. Also here: the error/CUDA-check helpers, the
// device arena, and MRG32k3a transition-matrix powers.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"
#include "kernels.cuh"

namespace ffea {
namespace host {

inline thread_local std::string g_last_error;

inline int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? FFEA_GPU_ENOMEM : FFEA_GPU_ECUDA;
}

#define CK(call)                                         \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// mesoDimensions, include/dimensions.h:30-41
constexpr double MESO_LENGTH = 1.7e-10;
constexpr double MESO_ENERGY = 4.141945559999999e-21;
constexpr double MESO_MASS = 1.994307387553024e-26;
constexpr double MESO_VOLUME = 4.913e-30;
constexpr double MESO_TIME = 3.7302915560886126e-13;
constexpr double MESO_PRESSURE = 8.4305832688784826e8;
constexpr double FFEA_PI = 3.141592653589793238462643383279502884197169399375105820974944592307816406286208998628034825342117067982148;

// ---------------------------------------------------------------------------
// MRG32k3a transition-matrix powers (host)
// ---------------------------------------------------------------------------
struct Mat3 {
    uint64_t m[3][3];
};

inline Mat3 mat_mul(const Mat3 &A, const Mat3 &B, uint64_t mod) {
    Mat3 C{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            uint64_t s = 0;
            for (int k = 0; k < 3; ++k) s = (s + (A.m[i][k] % mod) * (B.m[k][j] % mod) % mod) % mod;
            C.m[i][j] = s;
        }
    return C;
}

inline Mat3 mat_pow(Mat3 A, uint64_t n, uint64_t mod) {
    Mat3 R{};
    for (int i = 0; i < 3; ++i) R.m[i][i] = 1;
    while (n) {
        if (n & 1) R = mat_mul(A, R, mod);
        A = mat_mul(A, A, mod);
        n >>= 1;
    }
    return R;
}

inline const Mat3 MRG_A1 = {{{0, 1, 0}, {0, 0, 1}, {MRG_M1 - 810728ull, 1403580ull, 0}}};
inline const Mat3 MRG_A2 = {{{0, 1, 0}, {0, 0, 1}, {MRG_M2 - 1370589ull, 0, 527612ull}}};

inline MrgJump to_jump(const Mat3 &a, const Mat3 &b) {
    MrgJump J;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            J.a[3 * i + j] = (uint32_t)a.m[i][j];
            J.b[3 * i + j] = (uint32_t)b.m[i][j];
        }
    return J;
}

// CheckSeed (src/RngStream.cpp:224): components below m1 / m2, neither triple all zero
inline bool valid_seed(const uint32_t s[6]) {
    for (int i = 0; i < 3; ++i)
        if (s[i] >= MRG_M1) return false;
    for (int i = 3; i < 6; ++i)
        if (s[i] >= MRG_M2) return false;
    if (s[0] == 0 && s[1] == 0 && s[2] == 0) return false;
    if (s[3] == 0 && s[4] == 0 && s[5] == 0) return false;
    return true;
}

inline MrgJump jump_pow(uint64_t n) { return to_jump(mat_pow(MRG_A1, n, MRG_M1), mat_pow(MRG_A2, n, MRG_M2)); }

// ---------------------------------------------------------------------------
// device memory owned by a blob
// ---------------------------------------------------------------------------
struct Arena {
    std::vector<void *> ptrs;
    ~Arena() { clear(); }
    void clear() {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
    }
    template <class T>
    cudaError_t alloc(T **out, size_t n) {
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        ptrs.push_back(p);
        *out = static_cast<T *>(p);
        return cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
    }
    template <class T>
    cudaError_t upload(T **out, const std::vector<T> &v) {
        cudaError_t e = alloc(out, v.size());
        if (e != cudaSuccess || v.empty()) return e;
        return cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    }
};

// ---------------------------------------------------------------------------
// host description built once from the mesh
// ---------------------------------------------------------------------------
struct HostModel {
    int n_all = 0, N = 0, T = 0;
    std::vector<int> lin_of;       // n_all -> vertex index or -1
    std::vector<int> node_of;      // N -> original node
    std::vector<int> mid_nodes;    // original indices of midpoint nodes
    std::vector<int> mid_a, mid_b; // their edge ends (vertex indices)
    std::vector<int> tets10;       // original topology
    std::vector<int> tet4;         // T*4 vertex indices
    std::vector<double> pos;       // 3*N meso
    std::vector<double> rho, A, B, G, E, vol0, last_det, jinv; // per element (jinv 9*T row-major)
    std::vector<int> pinned;       // N flags
    std::vector<int> pinned_all;   // n_all flags
    std::vector<double> drag;      // N (stokes drag), empty if calc_stokes == 0
    std::vector<double> drag_all;  // n_all
    // incidence
    std::vector<int> inc_ptr, inc;
    // pattern (SELL-32 3x3 blocks)
    int nslices = 0;
    long long nslots = 0;
    std::vector<int> slice_ptr, rowlen, bcol, diagk;
    std::vector<int> grp_slice;  // slice of each group of 32 slots
    std::vector<std::vector<int>> nbr;  // sorted neighbours per vertex
    std::vector<int> src_ptr;
    std::vector<unsigned> src;
    // mass matrix values (solver CG), SELL scalar over the same pattern; lumped inverse masses
    std::vector<double> mass_sell, inv_mass;
    // Stokes noise: per vertex, the linearise events of its elements (element order), each holding up to
    // three midpoints (index into mid_nodes, -1 once the midpoint's force has been moved)
    std::vector<int> lin_ptr;
    std::vector<int> lin_ev;  // 4 per event (the fourth unused)
};

// calc_shape_function_derivatives_and_volume's determinant and mat3_invert, in the reference's order
inline void rest_state(HostModel &h) {
    const int T = h.T;
    h.vol0.assign(T, 0.0);
    h.last_det.assign(T, 0.0);
    h.jinv.assign(9 * (size_t)T, 0.0);
    for (int e = 0; e < T; ++e) {
        const int *t = &h.tet4[4 * (size_t)e];
        double m[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) m[r][c] = h.pos[3 * (size_t)t[r + 1] + c] - h.pos[3 * (size_t)t[0] + c];
        double *inv = &h.jinv[9 * (size_t)e];
        inv[0] = m[2][2] * m[1][1] - m[2][1] * m[1][2];
        inv[1] = m[2][1] * m[0][2] - m[2][2] * m[0][1];
        inv[2] = m[1][2] * m[0][1] - m[1][1] * m[0][2];
        inv[3] = m[2][0] * m[1][2] - m[2][2] * m[1][0];
        inv[4] = m[2][2] * m[0][0] - m[2][0] * m[0][2];
        inv[5] = m[1][0] * m[0][2] - m[1][2] * m[0][0];
        inv[6] = m[2][1] * m[1][0] - m[2][0] * m[1][1];
        inv[7] = m[2][0] * m[0][1] - m[2][1] * m[0][0];
        inv[8] = m[1][1] * m[0][0] - m[1][0] * m[0][1];
        double det = m[0][0] * inv[0] + m[1][0] * inv[1] + m[2][0] * inv[2];
        // calc_shape_function_derivatives_and_volume stores this det as last_det and |det|/6 as vol
        h.last_det[e] = det;
        h.vol0[e] = (1.0 / 6.0) * fabs(det);
        const double id = 1.0 / det;
        for (int k = 0; k < 9; ++k) inv[k] *= id;
    }
}

// The vertex side of Blob::linearise_force, replayed once: per vertex, in element order, the (up to three)
// midpoints whose force the vertex receives (a midpoint's force moves through the first element holding it).
inline void build_linearise_events(HostModel &h) {
    const int n = h.n_all, N = h.N, T = h.T;
    // Blob::linearise_force (src/Blob.cpp:781-799) walks the elements in order: each vertex gains half of
    // the three midpoints at it, then the element's six midpoints are zeroed, so a midpoint's force goes
    // to its edge ends once, through the first element that holds it
    static const int at_vertex[4][3] = {{4, 5, 6}, {4, 7, 8}, {5, 7, 9}, {6, 8, 9}};
    std::vector<int> mid_id(n, -1);
    for (size_t m = 0; m < h.mid_nodes.size(); ++m) mid_id[h.mid_nodes[m]] = (int)m;
    std::vector<char> moved(n, 0);
    std::vector<std::vector<int>> ev(N);
    for (int e = 0; e < T; ++e) {
        const int *t = &h.tets10[10 * (size_t)e];
        for (int j = 0; j < 4; ++j) {
            int q[3];
            bool live = false;
            for (int k = 0; k < 3; ++k) {
                const int x = t[at_vertex[j][k]];
                q[k] = moved[x] ? -1 : mid_id[x];
                live = live || q[k] >= 0;
            }
            if (!live) continue;
            auto &v = ev[h.lin_of[t[j]]];
            v.insert(v.end(), {q[0], q[1], q[2], -1});
        }
        for (int k = 4; k < 10; ++k) moved[t[k]] = 1;
    }
    h.lin_ptr.assign(N + 1, 0);
    for (int a = 0; a < N; ++a) h.lin_ptr[a + 1] = h.lin_ptr[a] + (int)ev[a].size() / 4;
    h.lin_ev.clear();
    h.lin_ev.reserve(4 * (size_t)h.lin_ptr[N]);
    for (int a = 0; a < N; ++a) h.lin_ev.insert(h.lin_ev.end(), ev[a].begin(), ev[a].end());
}

// The mixed element kernel's thread-block lists: for each block of `cta` consecutive elements, its distinct
// vertices in ascending order (cta_nodes[cta_ptr[c] .. cta_ptr[c + 1])), each element's four vertices as indices
// into its block's list (loc, 4 per element), and where each (block, vertex) force sum goes: perm[p] for the p-th
// list entry, such that a vertex's sums lie together, in block order, at [part_ptr[a], part_ptr[a + 1]).
// The block's own incidence: its 4 x (elements) (element, slot) pairs, coded 4 el + slot with el the element's
// index in the block, sorted by vertex and, for each vertex, by element (inc_local[4 cta c ..]); the p-th list
// entry's run starts at inc_start[p] within its block's part and ends where the next entry's starts (the block's
// last entry at 4 x its elements).
struct CtaLists {
    std::vector<int> cta_ptr, cta_nodes, perm, part_ptr;
    std::vector<uint16_t> loc, inc_local, inc_start;
};

inline void build_cta_lists(const HostModel &h, int cta, CtaLists &o) {
    const int T = h.T, N = h.N, nc = (T + cta - 1) / cta;
    o.cta_ptr.assign(nc + 1, 0);
    o.cta_nodes.clear();
    o.inc_local.clear();
    o.inc_start.clear();
    o.loc.assign(4 * (size_t)T, 0);
    std::vector<int> list;
    for (int c = 0; c < nc; ++c) {
        const int e0 = c * cta, e1 = std::min(T, e0 + cta);
        list.assign(h.tet4.begin() + 4 * (size_t)e0, h.tet4.begin() + 4 * (size_t)e1);
        std::sort(list.begin(), list.end());
        list.erase(std::unique(list.begin(), list.end()), list.end());
        for (size_t k = 4 * (size_t)e0; k < 4 * (size_t)e1; ++k)
            o.loc[k] = (uint16_t)(std::lower_bound(list.begin(), list.end(), h.tet4[k]) - list.begin());
        // the block's incidence, by vertex then element (a counting sort over the local vertex indices)
        std::vector<int> cnt(list.size() + 1, 0);
        for (size_t k = 4 * (size_t)e0; k < 4 * (size_t)e1; ++k) cnt[o.loc[k] + 1]++;
        for (size_t i = 0; i < list.size(); ++i) cnt[i + 1] += cnt[i];
        for (size_t i = 0; i < list.size(); ++i) o.inc_start.push_back((uint16_t)cnt[i]);
        std::vector<uint16_t> blk(4 * (size_t)cta, 0);
        for (size_t k = 4 * (size_t)e0; k < 4 * (size_t)e1; ++k) blk[cnt[o.loc[k]]++] = (uint16_t)(k - 4 * (size_t)e0);
        o.inc_local.insert(o.inc_local.end(), blk.begin(), blk.end());
        o.cta_nodes.insert(o.cta_nodes.end(), list.begin(), list.end());
        o.cta_ptr[c + 1] = (int)o.cta_nodes.size();
    }
    o.part_ptr.assign(N + 1, 0);
    for (int a : o.cta_nodes) o.part_ptr[a + 1]++;
    for (int a = 0; a < N; ++a) o.part_ptr[a + 1] += o.part_ptr[a];
    std::vector<int> fill(o.part_ptr.begin(), o.part_ptr.end() - 1);
    o.perm.resize(o.cta_nodes.size());
    for (size_t q = 0; q < o.cta_nodes.size(); ++q) o.perm[q] = fill[o.cta_nodes[q]]++;
}

inline int build_model(const ffea_gpu_mesh *mesh, const ffea_gpu_params *p, HostModel &h) {
    const int n = mesh->num_nodes, T = mesh->num_elements;
    if (n <= 0 || T <= 0 || mesh->num_pinned < 0 || !mesh->pos || !mesh->tets || !mesh->rho || !mesh->A ||
        !mesh->B || !mesh->G || !mesh->E) {
        g_last_error = "empty mesh or missing arrays";
        return FFEA_GPU_EINPUT;
    }
    if (T >= (1 << 28)) {
        g_last_error = "too many elements (limit 2^28)";
        return FFEA_GPU_EINPUT;
    }
    if (p->calc_stokes == 1 && !mesh->stokes_radius) {
        g_last_error = "calc_stokes needs stokes_radius";
        return FFEA_GPU_EINPUT;
    }
    h.n_all = n;
    h.T = T;
    h.tets10.assign(mesh->tets, mesh->tets + 10 * (size_t)T);
    std::vector<char> is_v(n, 0), is_m(n, 0);
    for (int e = 0; e < T; ++e)
        for (int s = 0; s < 10; ++s) {
            const int x = h.tets10[10 * (size_t)e + s];
            if (x < 0 || x >= n) {
                g_last_error = "element references an out of bounds node index";
                return FFEA_GPU_EINPUT;
            }
            (s < 4 ? is_v : is_m)[x] = 1;
        }
    h.lin_of.assign(n, -1);
    for (int i = 0; i < n; ++i) {
        if (is_v[i] && is_m[i]) {
            g_last_error = "a node is both an element vertex and an edge midpoint (unsupported topology)";
            return FFEA_GPU_EINPUT;
        }
        if (!is_v[i] && !is_m[i]) {
            g_last_error = "a node belongs to no element";
            return FFEA_GPU_EINPUT;
        }
        if (is_v[i]) {
            h.lin_of[i] = (int)h.node_of.size();
            h.node_of.push_back(i);
        }
    }
    h.N = (int)h.node_of.size();
    const int N = h.N;
    // midpoints: ends from the first element holding them (linearise_element, src/tetra_element_linear.cpp:553-577)
    static const int mid_pair[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    std::vector<int> mid_seen(n, 0);
    for (int e = 0; e < T; ++e)
        for (int s = 4; s < 10; ++s) {
            const int x = h.tets10[10 * (size_t)e + s];
            if (mid_seen[x]) continue;
            mid_seen[x] = 1;
            h.mid_nodes.push_back(x);
            h.mid_a.push_back(h.lin_of[h.tets10[10 * (size_t)e + mid_pair[s - 4][0]]]);
            h.mid_b.push_back(h.lin_of[h.tets10[10 * (size_t)e + mid_pair[s - 4][1]]]);
        }
    h.tet4.resize(4 * (size_t)T);
    for (int e = 0; e < T; ++e)
        for (int s = 0; s < 4; ++s) h.tet4[4 * (size_t)e + s] = h.lin_of[h.tets10[10 * (size_t)e + s]];
    h.pos.resize(3 * (size_t)N);
    for (int k = 0; k < N; ++k)
        for (int c = 0; c < 3; ++c) h.pos[3 * (size_t)k + c] = mesh->pos[3 * (size_t)h.node_of[k] + c];
    h.rho.assign(mesh->rho, mesh->rho + T);
    h.A.assign(mesh->A, mesh->A + T);
    h.B.assign(mesh->B, mesh->B + T);
    h.G.assign(mesh->G, mesh->G + T);
    h.E.assign(mesh->E, mesh->E + T);
    h.pinned_all.assign(n, 0);
    h.pinned.assign(N, 0);
    for (int k = 0; k < mesh->num_pinned; ++k) {
        const int x = mesh->pinned[k];
        if (x < 0 || x >= n) {
            g_last_error = "pinned node index out of bounds";
            return FFEA_GPU_EINPUT;
        }
        h.pinned_all[x] = 1;
        if (h.lin_of[x] >= 0) h.pinned[h.lin_of[x]] = 1;
    }
    if (p->calc_stokes == 1) {
        // Blob::init: stokes_drag = 6 pi eta r (src/Blob.cpp:262-268)
        h.drag_all.resize(n);
        for (int i = 0; i < n; ++i) h.drag_all[i] = 6.0 * FFEA_PI * p->stokes_visc * mesh->stokes_radius[i];
        h.drag.resize(N);
        for (int k = 0; k < N; ++k) h.drag[k] = h.drag_all[h.node_of[k]];
    }
    if (p->calc_stokes == 1 && p->calc_noise == 1) build_linearise_events(h);
    rest_state(h);
    // incidence: element order, vertex slots (Blob::calculate_node_element_connectivity)
    h.inc_ptr.assign(N + 1, 0);
    for (int e = 0; e < T; ++e)
        for (int s = 0; s < 4; ++s) h.inc_ptr[h.tet4[4 * (size_t)e + s] + 1]++;
    for (int k = 0; k < N; ++k) h.inc_ptr[k + 1] += h.inc_ptr[k];
    h.inc.resize(4 * (size_t)T);
    {
        std::vector<int> fill(N, 0);
        for (int e = 0; e < T; ++e)
            for (int s = 0; s < 4; ++s) {
                const int a = h.tet4[4 * (size_t)e + s];
                h.inc[h.inc_ptr[a] + fill[a]++] = 4 * e + s;
            }
    }
    // neighbours: unpinned vertex pairs sharing an element; pinned rows keep only their diagonal
    h.nbr.assign(N, {});
    for (int e = 0; e < T; ++e) {
        const int *t = &h.tet4[4 * (size_t)e];
        for (int a = 0; a < 4; ++a) {
            if (h.pinned[t[a]]) continue;
            for (int b = 0; b < 4; ++b)
                if (!h.pinned[t[b]]) h.nbr[t[a]].push_back(t[b]);
        }
    }
    for (int k = 0; k < N; ++k) {
        auto &v = h.nbr[k];
        if (h.pinned[k]) v.assign(1, k);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    // SELL-32 slices
    h.nslices = (N + 31) / 32;
    h.slice_ptr.assign(h.nslices + 1, 0);
    h.rowlen.assign(N, 0);
    h.diagk.assign(N, 0);
    for (int s = 0; s < h.nslices; ++s) {
        int w = 0;
        for (int l = 0; l < 32 && 32 * s + l < N; ++l) w = std::max<int>(w, (int)h.nbr[32 * s + l].size());
        h.slice_ptr[s + 1] = h.slice_ptr[s] + 32 * w;
    }
    h.nslots = h.slice_ptr[h.nslices];
    h.grp_slice.assign((size_t)(h.nslots / 32), 0);
    for (int s = 0; s < h.nslices; ++s)
        for (int gidx = h.slice_ptr[s] / 32; gidx < h.slice_ptr[s + 1] / 32; ++gidx) h.grp_slice[gidx] = s;
    if (h.nslots >= (1ll << 31)) {
        g_last_error = "matrix too large for 32-bit slot indices";
        return FFEA_GPU_EINPUT;
    }
    h.bcol.assign(h.nslots, 0);
    for (int a = 0; a < N; ++a) {
        const int s = a >> 5, lane = a & 31;
        const auto &v = h.nbr[a];
        h.rowlen[a] = (int)v.size();
        const int w = (h.slice_ptr[s + 1] - h.slice_ptr[s]) / 32;
        for (int k = 0; k < w; ++k) h.bcol[h.slice_ptr[s] + 32 * k + lane] = k < (int)v.size() ? v[k] : a;
        h.diagk[a] = (int)(std::lower_bound(v.begin(), v.end(), a) - v.begin());
    }
    // assembly sources per slot, element order (the registration order of NoMassCGSolver::init)
    auto slot_of = [&](int a, int b) -> long long {
        const auto &v = h.nbr[a];
        const int k = (int)(std::lower_bound(v.begin(), v.end(), b) - v.begin());
        return (long long)h.slice_ptr[a >> 5] + 32 * k + (a & 31);
    };
    h.src_ptr.assign(h.nslots + 1, 0);
    for (int e = 0; e < T; ++e) {
        const int *t = &h.tet4[4 * (size_t)e];
        for (int a = 0; a < 4; ++a) {
            if (h.pinned[t[a]]) continue;
            for (int b = 0; b < 4; ++b)
                if (!h.pinned[t[b]]) h.src_ptr[slot_of(t[a], t[b]) + 1]++;
        }
    }
    for (int a = 0; a < N; ++a)
        if (h.pinned[a]) h.src_ptr[slot_of(a, a) + 1]++;
    for (long long k = 0; k < h.nslots; ++k) h.src_ptr[k + 1] += h.src_ptr[k];
    h.src.assign(h.src_ptr[h.nslots], 0u);
    {
        std::vector<int> fill(h.nslots, 0);
        for (int a = 0; a < N; ++a)
            if (h.pinned[a]) {
                const long long k = slot_of(a, a);
                h.src[h.src_ptr[k] + fill[k]++] = SRC_IDENTITY;
            }
        for (int e = 0; e < T; ++e) {
            const int *t = &h.tet4[4 * (size_t)e];
            for (int a = 0; a < 4; ++a) {
                if (h.pinned[t[a]]) continue;
                for (int b = 0; b < 4; ++b) {
                    if (h.pinned[t[b]]) continue;
                    const long long k = slot_of(t[a], t[b]);
                    h.src[h.src_ptr[k] + fill[k]++] = ((unsigned)e << 4) | ((unsigned)a << 2) | (unsigned)b;
                }
            }
        }
    }
    // ConjugateGradientSolver::init mass matrix (src/ConjugateGradientSolver.cpp:78-115), vertex rows
    if (p->solver == FFEA_GPU_CG) {
        h.mass_sell.assign(h.nslots, 0.0);
        std::vector<char> set_one(h.nslots, 0);
        for (int e = 0; e < T; ++e) {
            const int *t = &h.tet4[4 * (size_t)e];
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) {
                    const int ni = t[i], nj = t[j];
                    if (!h.pinned[ni] && !h.pinned[nj]) {
                        const long long k = slot_of(ni, nj);
                        if (i == j) h.mass_sell[k] += .1 * h.rho[e] * h.vol0[e];
                        else h.mass_sell[k] += .05 * h.rho[e] * h.vol0[e];
                    } else if (i == j) {
                        h.mass_sell[slot_of(ni, nj)] = 1;
                    }
                }
        }
    }
    // MassLumpedSolver::init (src/MassLumpedSolver.cpp:27-62)
    if (p->solver == FFEA_GPU_MASSLUMPED) {
        h.inv_mass.assign(N, 0.0);
        for (int e = 0; e < T; ++e)
            for (int s = 0; s < 4; ++s) h.inv_mass[h.tet4[4 * (size_t)e + s]] += .25 * h.rho[e] * h.vol0[e];
        for (int a = 0; a < N; ++a) {
            if (h.pinned[a]) h.inv_mass[a] = 1.0;
            h.inv_mass[a] = 1.0 / h.inv_mass[a];
        }
    }
    return FFEA_GPU_OK;
}

template <class R>
std::vector<R> cast_vec(const std::vector<double> &v) {
    return std::vector<R>(v.begin(), v.end());
}

// Rigid motions v_a = t + omega x (x_a - x_c) that leave every pinned vertex at rest: the null
// space of the viscosity matrix when there is no Stokes drag (mixed-path CG deflation). Returns the
// mode coefficients (t, omega) row-wise in modes[6*k..6*k+5].
// Vertex rows [row0, row0 + nrows) (default: all) are one blob of a batch.
// the rigid modes about a given reference point xc (see rigid_modes); reads only the pinned rows' positions
inline int rigid_modes_about(const HostModel &h, const ffea_gpu_params &p, const double xc[3], double modes[36],
                             int row0, int nrows);

// The rigid-body modes the mixed CG deflates, about the centroid xc of rows [row0, row0 + nrows): all six
// without pins, those that keep every pinned vertex at rest with pins, none with Stokes drag.
inline int rigid_modes(const HostModel &h, const ffea_gpu_params &p, double xc[3], double modes[36], int row0 = 0,
                       int nrows = -1) {
    if (nrows < 0) nrows = h.N - row0;
    const int row1 = row0 + nrows;
    xc[0] = xc[1] = xc[2] = 0.0;
    for (int a = row0; a < row1; ++a)
        for (int c = 0; c < 3; ++c) xc[c] += h.pos[3 * (size_t)a + c];
    for (int c = 0; c < 3; ++c) xc[c] /= std::max(nrows, 1);
    return rigid_modes_about(h, p, xc, modes, row0, nrows);
}

inline int rigid_modes_about(const HostModel &h, const ffea_gpu_params &p, const double xc[3], double modes[36],
                             int row0, int nrows) {
    if (nrows < 0) nrows = h.N - row0;
    const int row1 = row0 + nrows;
    if (p.calc_stokes == 1) return 0;
    // M = sum over pinned vertices of C^T C, C = [I | -[d]x]
    double M[6][6] = {};
    int npin = 0;
    for (int a = row0; a < row1; ++a) {
        if (!h.pinned[a]) continue;
        ++npin;
        const double d[3] = {h.pos[3 * (size_t)a] - xc[0], h.pos[3 * (size_t)a + 1] - xc[1],
                             h.pos[3 * (size_t)a + 2] - xc[2]};
        double C[3][6] = {{1, 0, 0, 0, d[2], -d[1]}, {0, 1, 0, -d[2], 0, d[0]}, {0, 0, 1, d[1], -d[0], 0}};
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j)
                for (int k = 0; k < 3; ++k) M[i][j] += C[k][i] * C[k][j];
    }
    double V[6][6] = {};
    for (int i = 0; i < 6; ++i) V[i][i] = 1.0;
    if (npin > 0) {  // cyclic Jacobi eigen-decomposition of the 6x6 symmetric M
        for (int sweep = 0; sweep < 100; ++sweep) {
            double off = 0.0;
            for (int i = 0; i < 6; ++i)
                for (int j = i + 1; j < 6; ++j) off += M[i][j] * M[i][j];
            if (off < 1e-30) break;
            for (int i = 0; i < 6; ++i)
                for (int j = i + 1; j < 6; ++j) {
                    if (fabs(M[i][j]) < 1e-300) continue;
                    const double th = 0.5 * atan2(2 * M[i][j], M[j][j] - M[i][i]);
                    const double c = cos(th), sn = sin(th);
                    for (int k = 0; k < 6; ++k) {
                        const double a = M[k][i], b = M[k][j];
                        M[k][i] = c * a - sn * b;
                        M[k][j] = sn * a + c * b;
                    }
                    for (int k = 0; k < 6; ++k) {
                        const double a = M[i][k], b = M[j][k];
                        M[i][k] = c * a - sn * b;
                        M[j][k] = sn * a + c * b;
                    }
                    for (int k = 0; k < 6; ++k) {
                        const double a = V[k][i], b = V[k][j];
                        V[k][i] = c * a - sn * b;
                        V[k][j] = sn * a + c * b;
                    }
                }
        }
    }
    double emax = 0.0;
    for (int i = 0; i < 6; ++i) emax = std::max(emax, fabs(M[i][i]));
    int k = 0;
    for (int i = 0; i < 6; ++i) {
        if (npin > 0 && fabs(M[i][i]) > 1e-9 * std::max(emax, 1.0)) continue;
        for (int j = 0; j < 6; ++j) modes[6 * k + j] = V[j][i];
        ++k;
    }
    return k;
}

// V[r][c] of the element viscosity matrix, same evaluation as the device's visc_entry
inline double host_visc_entry(const double *dpsi, double A, double B, double vol, int r, int c) {
    if (r > c) std::swap(r, c);
    const int i = r >> 2, a = r & 3, j = c >> 2, b = c & 3;
    if (i == j) {
        const double t = dpsi[4 * i + a] * dpsi[4 * i + b] * (A + B);
        const double d2 = (dpsi[a] * dpsi[b] + dpsi[4 + a] * dpsi[4 + b] + dpsi[8 + a] * dpsi[8 + b]);
        return (t + d2 * A) * vol;
    }
    if (a == b) return ((B + A) * (dpsi[4 * i + a] * dpsi[4 * j + a])) * vol;
    return (B * (dpsi[4 * i + a] * dpsi[4 * j + b]) + A * (dpsi[4 * i + b] * dpsi[4 * j + a])) * vol;
}

}  // namespace host
}  // namespace ffea
