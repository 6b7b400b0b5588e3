// ctforces_device.h -- device arrays of the constant forces (Blob::apply_ctforces, src/Blob.cpp:1676-1743) for
// the node kernels (gather_kernel, gather_mixed_kernel, mid_force_kernel), the rotational kernel and the
// surface kernels: one blob's, or a replica batch's with every blob's forces in the concatenated numbering.
#pragma once

#include <string>
#include <vector>

#include "ctforces.h"
#include "engine.h"
#include "host_model.h"

namespace ffea {

struct CtfDevice {
    host::Arena mem;
    double *node = nullptr, *mid = nullptr, *ff = nullptr;  // 3 per vertex / midpoint / face
    int *vface_ptr = nullptr, *vface = nullptr, *mface_ptr = nullptr, *mface = nullptr;
    SurfArgs surf{};
    RotArgs rot{};
    bool mid_force = false;  // some midpoint carries a constant force (the linearise replay is needed)
    bool any = false;        // any constant force at all

    void release() {
        mem.clear();
        node = mid = ff = nullptr;
        vface_ptr = vface = mface_ptr = mface = nullptr;
        surf = SurfArgs{};
        rot = RotArgs{};
        mid_force = any = false;
    }

    // cm over h's reference numbering (h.n_all nodes); px..pz the device positions the per-step kernels read. On
    // an error nothing is left half built: the device holds no constant forces.
    cudaError_t build(const host::HostModel &h, const host::CtfModel &cm, const double *px, const double *py,
                      const double *pz, const DevStatus *st) {
        const cudaError_t e = build_arrays(h, cm, px, py, pz, st);
        if (e != cudaSuccess) release();
        return e;
    }

  private:
    cudaError_t build_arrays(const host::HostModel &h, const host::CtfModel &cm, const double *px, const double *py,
                             const double *pz, const DevStatus *st) {
        release();
        const int N = h.N, M = (int)h.mid_nodes.size(), n = h.n_all;
        std::vector<int> mid_id(n, -1);
        for (int m = 0; m < M; ++m) mid_id[h.mid_nodes[m]] = m;
        bool any_lin = false;
        std::vector<double> vn(3 * (size_t)N, 0.0), vm(3 * (size_t)std::max(M, 1), 0.0);
        for (int k = 0; k < N; ++k)
            for (int c = 0; c < 3; ++c) vn[3 * (size_t)k + c] = cm.lin[3 * (size_t)h.node_of[k] + c];
        for (int m = 0; m < M; ++m) {
            for (int c = 0; c < 3; ++c) vm[3 * (size_t)m + c] = cm.lin[3 * (size_t)h.mid_nodes[m] + c];
            mid_force = mid_force || cm.has_lin[h.mid_nodes[m]] || !cm.rot[h.mid_nodes[m]].empty();
        }
        for (int i = 0; i < n; ++i) any_lin = any_lin || cm.has_lin[i] || !cm.rot[i].empty();
        // rotational forces: the nodes carrying them, in vertex then midpoint order, with their forces in file
        // order
        std::vector<int> rv_row, rv_ptr(1, 0), rm_idx, rm_ptr(1, 0);
        std::vector<RotEntry> rent;
        auto add_rot = [&](int x) {
            for (const host::RotCtf &r : cm.rot[x]) {
                RotEntry e{};
                e.F = r.F;
                e.torque = r.torque;
                for (int c = 0; c < 3; ++c) { e.p[c] = r.p[c]; e.d[c] = r.d[c]; }
                rent.push_back(e);
            }
        };
        for (int k = 0; k < N; ++k)
            if (!cm.rot[h.node_of[k]].empty()) {
                rv_row.push_back(k);
                add_rot(h.node_of[k]);
                rv_ptr.push_back((int)rent.size());
            }
        for (int m = 0; m < M; ++m)
            if (!cm.rot[h.mid_nodes[m]].empty()) {
                rm_idx.push_back(m);
                add_rot(h.mid_nodes[m]);
                rm_ptr.push_back((int)rent.size() - rv_ptr.back());
            }
        cudaError_t e;
        if (any_lin) {
            if ((e = mem.upload(&node, vn)) != cudaSuccess) return e;
            if (mid_force && (e = mem.upload(&mid, vm)) != cudaSuccess) return e;
        }
        if (!rent.empty()) {
            // the static linear sums stay as they are; the node kernels read copies the rotational kernel
            // rewrites for its nodes every step
            double *lin_v = node, *lin_m = mid;
            if ((e = mem.upload(&node, vn)) != cudaSuccess) return e;
            if (mid_force && (e = mem.upload(&mid, vm)) != cudaSuccess) return e;
            int *d_vrow, *d_vptr, *d_midx, *d_mptr, *d_ma, *d_mb;
            RotEntry *d_ent;
            if (rv_row.empty()) rv_row.push_back(0);
            if (rm_idx.empty()) rm_idx.push_back(0);
            std::vector<int> ma(h.mid_a), mb(h.mid_b);
            if (ma.empty()) { ma.push_back(0); mb.push_back(0); }
            if ((e = mem.upload(&d_vrow, rv_row)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_vptr, rv_ptr)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_midx, rm_idx)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_mptr, rm_ptr)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_ent, rent)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_ma, ma)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_mb, mb)) != cudaSuccess) return e;
            rot.nv = (int)rv_ptr.size() - 1;
            rot.nm = (int)rm_ptr.size() - 1;
            rot.v_row = d_vrow; rot.v_ptr = d_vptr; rot.m_idx = d_midx; rot.m_ptr = d_mptr;
            rot.ent = d_ent;
            rot.ent_m = d_ent + rv_ptr.back();
            rot.mid_a = d_ma; rot.mid_b = d_mb;
            rot.px = px; rot.py = py; rot.pz = pz;
            rot.lin_v = lin_v; rot.lin_m = lin_m;
            rot.out_v = node; rot.out_m = mid;
            rot.st = st;
        }
        const int nsets = (int)cm.set_ptr.size() - 1;
        if (nsets > 0) {
            const int nf = (int)cm.face_nodes.size() / 3;
            std::vector<int2> corner(3 * (size_t)nf);
            for (int f = 0; f < nf; ++f)
                for (int k = 0; k < 3; ++k) {
                    const int x = cm.face_nodes[3 * (size_t)f + k];
                    corner[3 * (size_t)f + k] = h.lin_of[x] >= 0 ? make_int2(h.lin_of[x], h.lin_of[x])
                                                                 : make_int2(h.mid_a[mid_id[x]], h.mid_b[mid_id[x]]);
                }
            // sets holding each face (set order); faces holding each node (face order), forced faces only
            std::vector<std::vector<int>> fs(nf), vf(N), mf(M);
            for (int s2 = 0; s2 < nsets; ++s2)
                for (int k = cm.set_ptr[s2]; k < cm.set_ptr[s2 + 1]; ++k) fs[cm.set_faces[k]].push_back(s2);
            for (int f = 0; f < nf; ++f) {
                if (fs[f].empty()) continue;
                for (int k = 0; k < 3; ++k) {
                    const int x = cm.face_nodes[3 * (size_t)f + k];
                    if (h.lin_of[x] >= 0) vf[h.lin_of[x]].push_back(f);
                    else { mf[mid_id[x]].push_back(f); mid_force = true; }
                }
            }
            auto csr = [](const std::vector<std::vector<int>> &v, std::vector<int> &ptr, std::vector<int> &idx) {
                ptr.assign(v.size() + 1, 0);
                for (size_t i = 0; i < v.size(); ++i) ptr[i + 1] = ptr[i] + (int)v[i].size();
                idx.clear();
                for (const auto &x : v) idx.insert(idx.end(), x.begin(), x.end());
                if (idx.empty()) idx.push_back(0);
            };
            std::vector<int> fsp, fsi, vfp, vfi, mfp, mfi;
            csr(fs, fsp, fsi);
            csr(vf, vfp, vfi);
            csr(mf, mfp, mfi);
            int *d_set_ptr, *d_set_faces, *d_fsp, *d_fsi;
            int2 *d_corner;
            double *d_setF, *d_total;
            if ((e = mem.upload(&d_set_ptr, cm.set_ptr)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_set_faces, cm.set_faces)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_setF, cm.set_force)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_corner, corner)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_fsp, fsp)) != cudaSuccess) return e;
            if ((e = mem.upload(&d_fsi, fsi)) != cudaSuccess) return e;
            if ((e = mem.alloc(&d_total, (size_t)nsets)) != cudaSuccess) return e;
            if ((e = mem.alloc(&ff, 3 * (size_t)nf)) != cudaSuccess) return e;
            if ((e = mem.upload(&vface_ptr, vfp)) != cudaSuccess) return e;
            if ((e = mem.upload(&vface, vfi)) != cudaSuccess) return e;
            if (M > 0) {
                if ((e = mem.upload(&mface_ptr, mfp)) != cudaSuccess) return e;
                if ((e = mem.upload(&mface, mfi)) != cudaSuccess) return e;
            }
            surf.nsets = nsets;
            surf.nfaces = nf;
            surf.set_ptr = d_set_ptr; surf.set_faces = d_set_faces; surf.set_force = d_setF;
            surf.corner = d_corner;
            surf.face_set_ptr = d_fsp; surf.face_set = d_fsi;
            surf.px = px; surf.py = py; surf.pz = pz;
            surf.set_total = d_total; surf.ff = ff;
            surf.st = st;
        }
        any = any_lin || nsets > 0;
        return cudaSuccess;
    }

  public:
    void fill(NodeForces &sn) const {
        sn.node_ctf = node;
        sn.mid_ctf = mid;
        sn.vface_ptr = vface_ptr; sn.vface = vface;
        sn.mface_ptr = mface_ptr; sn.mface = mface;
        sn.ff = ff;
    }

    // the step's rotational and surface forces, before the node kernels read them
    cudaError_t launch(cudaStream_t s) const {
        cudaError_t e = cudaSuccess;
        if (rot.nv + rot.nm > 0 && (e = launch_rot_forces(rot, s)) != cudaSuccess) return e;
        if (surf.nsets > 0) e = launch_surface_forces(surf, s);
        return e;
    }
};

}  // namespace ffea
