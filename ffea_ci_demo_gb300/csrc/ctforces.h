// ctforces.h -- the reference's constant-force file (Blob::load_ctforces, src/Blob.cpp:2478-2805) for one blob:
// linear forces on nodes (CTF 1), rotational forces about an axis through a point (CTF 2), and linear forces
// spread over sets of surface faces in proportion to their areas (CTF 3). Host only.
#pragma once

#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace ffea {
namespace host {

constexpr double MESO_FORCE = 2.4364705882352941e-11;   // mesoDimensions::force (include/dimensions.h:37)
constexpr double MESO_LENGTH_CTF = 1.7e-10;             // mesoDimensions::length (include/dimensions.h:31)

// one rotational constant force (CTF 2) on one node: about the axis through p along the unit vector d,
// F times (r x d) ('f') or F / |r| times (r x d) ('t'), r from the node to its nearest point on the axis
struct RotCtf {
    double F;
    int torque;
    double p[3], d[3];
};

struct CtfModel {
    // CTF 1: per node of the reference numbering, the sum of its linear forces in file order (meso)
    std::vector<double> lin;
    std::vector<char> has_lin;
    // CTF 2: per node, its rotational forces in file order (the reference adds them after the linear ones)
    std::vector<std::vector<RotCtf>> rot;
    // CTF 3: surface faces (3 corner nodes, reference numbering), sets of faces with their force (meso)
    std::vector<int> face_nodes;
    std::vector<double> set_force;        // 3 per set
    std::vector<int> set_ptr, set_faces;  // the faces of each set, in file order
};

inline std::vector<std::string> ctf_lines(const std::string &fname, bool &ok) {
    std::vector<std::string> out;
    std::ifstream f(fname);
    ok = (bool)f;
    std::string line;
    bool in_comment = false;
    while (ok && std::getline(f, line)) {
        std::string keep;
        size_t i = 0;
        while (i < line.size()) {
            if (in_comment) {
                const size_t e = line.find("-->", i);
                if (e == std::string::npos) { i = line.size(); break; }
                in_comment = false;
                i = e + 3;
            } else {
                const size_t b = line.find("<!--", i);
                if (b == std::string::npos) { keep += line.substr(i); break; }
                keep += line.substr(i, b - i);
                in_comment = true;
                i = b + 4;
            }
        }
        const size_t a = keep.find_first_not_of(" \t\r\n");
        if (a == std::string::npos) continue;
        keep = keep.substr(a, keep.find_last_not_of(" \t\r\n") - a + 1);
        out.push_back(keep);
    }
    return out;
}

inline std::vector<std::string> ctf_split(const std::string &s) {
    std::istringstream is(s);
    std::vector<std::string> v;
    std::string w;
    while (is >> w) v.push_back(w);
    return v;
}

// F * d / |d| / mesoDimensions::force, as load_ctforces normalises and converts (src/Blob.cpp:2596-2606);
// false for a zero direction, which normalize refuses (include/mat_vec_fns_II.h:188-198)
inline bool ctf_force(double F, double d0, double d1, double d2, double out[3]) {
    double d[3] = {d0, d1, d2}, sum = 0;
    for (int i = 0; i < 3; ++i) sum += d[i] * d[i];
    if (sum == 0) return false;
    sum = std::sqrt(sum);
    for (int i = 0; i < 3; ++i) d[i] = d[i] / sum;
    for (int i = 0; i < 3; ++i) out[i] = F * d[i] / MESO_FORCE;
    return true;
}

// Reads the forces of blob `blob_index` (conformation 0). surf_file is needed when the file has surface forces.
inline int load_ctforces(const char *ctf_file, const char *surf_file, int blob_index, int n_all, CtfModel &m,
                         std::string &err) {
    bool ok = false;
    const std::vector<std::string> L = ctf_lines(ctf_file, ok);
    if (!ok) { err = std::string("cannot read ") + ctf_file; return 8; }
    if (L.size() < 4) { err = "ctforces file too short"; return 3; }
    int n_ct = 0, n_l = 0, n_r = 0, n_s = 0, at = 1;
    for (; at < 5 && at < (int)L.size(); ++at) {
        if (L[at].find(':') != std::string::npos) break;
        const auto w = ctf_split(L[at]);
        if (w.size() < 2) continue;
        const int v = atoi(w[1].c_str());
        if (w[0] == "num_ctforces") n_ct = v;
        else if (w[0] == "num_linear_forces") n_l = v;
        else if (w[0] == "num_rot_forces") n_r = v;
        else if (w[0] == "num_linear_surface_forces") n_s = v;
    }
    const int lines = n_ct + at + (n_l ? 1 : 0) + (n_r ? 1 : 0) + (n_s ? 1 : 0);
    if (n_ct != n_l + n_r + n_s || n_ct == 0 || lines != (int)L.size()) {
        err = "inconsistent ctforces header";
        return 3;
    }
    m.lin.assign(3 * (size_t)n_all, 0.0);
    m.has_lin.assign(n_all, 0);
    m.set_ptr.assign(1, 0);
    if (L[at].compare(0, 14, "linear forces:") == 0) ++at;
    else if (n_l > 0) { err = "expected 'linear forces:'"; return 3; }
    for (int i = at; i < at + n_l; ++i) {
        const auto w = ctf_split(L[i]);
        if (w.size() != 7) { err = "invalid linear force line: " + L[i]; return 3; }
        if (atoi(w[4].c_str()) != blob_index || atoi(w[5].c_str()) != 0) continue;
        double f[3];
        if (!ctf_force(atof(w[0].c_str()), atof(w[1].c_str()), atof(w[2].c_str()), atof(w[3].c_str()), f)) {
            err = "constant force with a zero direction";
            return 3;
        }
        auto add = [&](int n) {
            for (int c = 0; c < 3; ++c) m.lin[3 * (size_t)n + c] += f[c];
            m.has_lin[n] = 1;
        };
        if (w[6] == "all") {
            for (int n = 0; n < n_all; ++n) add(n);
        } else {
            const int n = atoi(w[6].c_str());
            if (n < 0 || n >= n_all) { err = "linear force on an out of range node"; return 3; }
            add(n);
        }
    }
    at += n_l;
    m.rot.assign(n_all, {});
    if (at < (int)L.size() && L[at].compare(0, 18, "rotational forces:") == 0) {
        ++at;
        // "F type px py pz dx dy dz blob conformation node|all" (src/Blob.cpp:2652-2730): F in N, the axis point
        // in m, type "p?" (an axis through a point; "n?" axes between nodes are not applied by the reference
        // either, src/Blob.cpp:1697-1705) and "?f" (F (r x d)) or "?t" (F/|r| (r x d))
        for (int i = at; i < at + n_r; ++i) {
            const auto w = ctf_split(L[i]);
            if (w.size() != 11) { err = "invalid rotational force line: " + L[i]; return 3; }
            if (atoi(w[8].c_str()) != blob_index || atoi(w[9].c_str()) != 0) continue;
            const std::string &type = w[1];
            if (type.size() < 2 || type[0] != 'p') {
                err = "rotational forces about an axis between nodes (type 'n') are not applied by the reference";
                return 3;
            }
            if (type[1] != 'f' && type[1] != 't') { err = "invalid rotational force type: " + type; return 3; }
            RotCtf r{};
            r.F = atof(w[0].c_str()) * (1. / MESO_FORCE);
            r.torque = type[1] == 't';
            double d[3] = {atof(w[5].c_str()), atof(w[6].c_str()), atof(w[7].c_str())}, sum = 0;
            for (int c = 0; c < 3; ++c) sum += d[c] * d[c];  // normalize, include/mat_vec_fns_II.h:188-198
            if (sum == 0) { err = "rotational force with a zero axis"; return 3; }
            sum = std::sqrt(sum);
            for (int c = 0; c < 3; ++c) {
                r.d[c] = d[c] / sum;
                r.p[c] = (1. / MESO_LENGTH_CTF) * atof(w[2 + c].c_str());  // resize(mdlm1, ctf_p)
            }
            if (w[10] == "all") {
                for (int n = 0; n < n_all; ++n) m.rot[n].push_back(r);
            } else {
                const int n = atoi(w[10].c_str());
                if (n < 0 || n >= n_all) { err = "rotational force on an out of range node"; return 3; }
                m.rot[n].push_back(r);
            }
        }
    } else if (n_r > 0) { err = "expected 'rotational forces:'"; return 3; }
    at += n_r;
    if (n_s > 0) {
        if (at >= (int)L.size() || L[at].compare(0, 22, "linear surface forces:") != 0) {
            err = "expected 'linear surface forces:'";
            return 3;
        }
        ++at;
        bool any = false;
        for (int i = at; i < at + n_s; ++i) {
            const auto w = ctf_split(L[i]);
            if (w.size() < 7) { err = "invalid surface force line: " + L[i]; return 3; }
            if (atoi(w[4].c_str()) != blob_index || atoi(w[5].c_str()) != 0) continue;
            if (w[6] == "all") { err = "surface forces on 'all' faces are refused by the reference too"; return 3; }
            any = true;
            double f[3];
            if (!ctf_force(atof(w[0].c_str()), atof(w[1].c_str()), atof(w[2].c_str()), atof(w[3].c_str()), f)) {
                err = "constant force with a zero direction";
                return 3;
            }
            m.set_force.insert(m.set_force.end(), f, f + 3);
            for (size_t j = 6; j < w.size(); ++j) m.set_faces.push_back(atoi(w[j].c_str()));
            m.set_ptr.push_back((int)m.set_faces.size());
        }
        if (any) {
            // Blob::load_surface (src/Blob.cpp:2089-2170): "element n0 n1 n2" per face
            if (!surf_file) { err = "surface constant forces need the blob's surface file"; return 3; }
            FILE *in = fopen(surf_file, "r");
            if (!in) { err = std::string("cannot read ") + surf_file; return 8; }
            char line[128];
            int nf = 0;
            if (!fgets(line, sizeof line, in) || fscanf(in, "num_surface_faces %d\n", &nf) != 1 ||
                !fgets(line, sizeof line, in)) {
                fclose(in);
                err = "malformed surface file";
                return 8;
            }
            m.face_nodes.resize(3 * (size_t)nf);
            for (int i = 0; i < nf; ++i) {
                int el, a, b, c;
                if (fscanf(in, "%d %d %d %d\n", &el, &a, &b, &c) != 4 || a < 0 || b < 0 || c < 0 || a >= n_all ||
                    b >= n_all || c >= n_all) {
                    fclose(in);
                    err = "malformed surface face";
                    return 8;
                }
                m.face_nodes[3 * (size_t)i] = a;
                m.face_nodes[3 * (size_t)i + 1] = b;
                m.face_nodes[3 * (size_t)i + 2] = c;
            }
            fclose(in);
            for (int f : m.set_faces)
                if (f < 0 || f >= nf) { err = "surface force on an out of range face"; return 3; }
        }
    }
    return 0;
}

// A model with no forces on n_all nodes.
inline void empty_ctforces(int n_all, CtfModel &m) {
    m = CtfModel{};
    m.lin.assign(3 * (size_t)n_all, 0.0);
    m.has_lin.assign(n_all, 0);
    m.rot.assign(n_all, {});
    m.set_ptr.assign(1, 0);
}

// Blob models side by side in one numbering (a replica batch): blob b's node i is node node_off[b] + i, its
// faces and sets follow those of the blobs before it.
inline void concat_ctforces(const std::vector<CtfModel> &parts, const std::vector<int> &node_off, CtfModel &out) {
    empty_ctforces(node_off.back(), out);
    for (size_t b = 0; b < parts.size(); ++b) {
        const CtfModel &m = parts[b];
        const int o = node_off[b], n = node_off[b + 1] - o;
        const int face0 = (int)out.face_nodes.size() / 3;
        for (int i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) out.lin[3 * (size_t)(o + i) + c] = m.lin[3 * (size_t)i + c];
            out.has_lin[o + i] = m.has_lin[i];
            out.rot[o + i] = m.rot[i];
        }
        for (int x : m.face_nodes) out.face_nodes.push_back(o + x);
        for (size_t s2 = 0; s2 + 1 < m.set_ptr.size(); ++s2) {
            for (int k = m.set_ptr[s2]; k < m.set_ptr[s2 + 1]; ++k) out.set_faces.push_back(face0 + m.set_faces[k]);
            out.set_ptr.push_back((int)out.set_faces.size());
            for (int c = 0; c < 3; ++c) out.set_force.push_back(m.set_force[3 * s2 + c]);
        }
    }
}

}  // namespace host
}  // namespace ffea
