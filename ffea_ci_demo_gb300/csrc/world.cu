// world.cu -- the .ffea script front-end: a World restricted to the blob-step path.
//
// It reads a reference .ffea script (FFEA_input_reader, src/FFEA_input_reader.cpp; World::init and
// read_and_build_system, src/World.cpp:54-620, 2300-2800), builds one GPU blob per <blob> from its
// structure files, places it (centroid, rotation, velocity, move into the simulation box), seeds the
// thermal stream from rng_seed, and runs World::run's step loop (src/World.cpp:1747-2059) for the
// blobs: every `check` steps the RNG state goes to the checkpoint file before the forces (.fcp,
// print_checkpoints :4546-4596) and, after them, the positions to the trajectory (.ftj,
// Blob::write_nodes_to_file, src/Blob.cpp:855-890) and the measurements to the measurement file (.fm,
// World::make_measurements / write_measurements_to_file :4598-4692). restart = 1 resumes from the
// checkpoint and the last complete trajectory frame (:300-425, :690-860).
//
// Constant forces (calc_ctforces = 1, <interactions><ctforces><ctforces_fname>) are loaded per blob
// with its surface file, as Blob::init does (src/Blob.cpp:188-190, read_and_build_system :2266-2290).
// Everything else outside the path is refused with FFEA_GPU_EINPUT and a message: surface-surface and
// steric interactions (calc_ssint, calc_steric must be set to 0), electrostatics, kinetics, springs,
// pre-computed potentials, rotational constant forces about an axis between two nodes (which the reference
// reads but never applies), rods, several conformations, STATIC/FROZEN blobs.
//
// The reference's threads each own a stream; this engine reproduces its single-thread order, in which
// one stream serves every blob: per step, the elements of blob 0, 1, ... draw 7 numbers each, then
// (Stokes noise) the nodes of blob 0, 1, ... draw 3 each. Each GPU blob starts its step on the stream
// advanced past the blobs before it and advances by the whole World's draws.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"
#include "blob_iface.h"
#include "host_model.h"

using namespace ffea;
using namespace ffea::host;

namespace {

// mesoDimensions derived units (include/dimensions.h:30-41)
constexpr double M_LENGTH = 1.7e-10;
constexpr double M_ENERGY = 4.141945559999999e-21;
constexpr double M_TIME = 3.7302915560886126e-13;
constexpr double M_VELOCITY = M_LENGTH / M_TIME;
constexpr double PI = 3.141592653589793238462643383279502884;

std::string trim(const std::string &s) {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

// FFEA_input_reader::file_to_lines: one tag per line, <!-- --> comments removed (across lines too)
bool script_lines(const std::string &fname, std::vector<std::string> &out) {
    std::ifstream f(fname);
    if (!f) return false;
    std::string line;
    bool in_comment = false;
    while (std::getline(f, line)) {
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
        keep = trim(keep);
        if (!keep.empty()) out.push_back(keep);
    }
    return true;
}

// FFEA_input_reader::parse_tag: "<key = value>" -> key, value (value empty for block tags)
void parse_tag(const std::string &t, std::string &key, std::string &val) {
    std::string s = t;
    if (!s.empty() && s.front() == '<') s.erase(0, 1);
    if (!s.empty() && s.back() == '>') s.pop_back();
    const size_t eq = s.find('=');
    key = trim(eq == std::string::npos ? s : s.substr(0, eq));
    val = eq == std::string::npos ? "" : trim(s.substr(eq + 1));
}

std::vector<double> tuple_values(std::string v) {
    for (char &c : v)
        if (c == '(' || c == ')' || c == ',') c = ' ';
    std::istringstream is(v);
    std::vector<double> out;
    double x;
    while (is >> x) out.push_back(x);
    return out;
}

std::string join_dir(const std::string &dir, const std::string &f) {
    if (f.empty() || f[0] == '/' || dir.empty()) return f;
    return dir + "/" + f;
}

struct BlobSpec {
    std::string nodes, topology, material, stokes, pin, surface, motion_state = "DYNAMIC";
    int solver = FFEA_GPU_NOMASS_CG;
    double scale = 0.0;  // metres per file unit
    bool set_centroid = false, set_velocity = false;
    int rotation_type = -1;  // 0: three angles (degrees), 1: matrix
    double centroid[3] = {0, 0, 0}, velocity[3] = {0, 0, 0}, rotation[9] = {0};
};

int fail(const std::string &msg) {
    g_last_error = msg;
    return FFEA_GPU_EINPUT;
}

}  // namespace

struct ffea_gpu_world {
    ffea_gpu_params p{};
    int precision = FFEA_GPU_FP64;
    long long num_steps = 100000000000ll, step_initial = 0;
    int check = 10000, restart = 0;
    long long rng_seed = 0;
    bool seed_set = false;
    int move_into_box = 1, es_N[3] = {-1, -1, -1}, calc_ctforces = 0;
    std::string ctforces_fname;
    double ssint_cutoff = 3e-9 / M_LENGTH;
    std::string script, dir, traj_fname, meas_fname, ockpt_fname, ickpt_fname;
    std::vector<BlobSpec> spec;
    std::vector<ffea_gpu_blob *> blobs;
    std::vector<int> n_all;
    bool mass_in_system = false;
    uint32_t stream[6] = {12345, 12345, 12345, 12345, 12345, 12345};
    FILE *traj = nullptr, *meas = nullptr;

    ~ffea_gpu_world() {
        if (traj) fclose(traj);
        if (meas) fclose(meas);
        for (auto *b : blobs) ffea_gpu_blob_destroy(b);
    }
    int read_params(const std::vector<std::string> &lines);
    int read_system(const std::vector<std::string> &lines);
    int build();
    int open_outputs();
    int restart_state();
    int write_frame(long long step);
    int write_measurement(long long step);
    int write_checkpoint();
    int run(long long *last_step);
};

// SimulationParams::assign over the keys of a <param> block (src/SimulationParams.cpp:245-760)
int ffea_gpu_world::read_params(const std::vector<std::string> &lines) {
    ffea_gpu_params_default(&p);
    p.solver = FFEA_GPU_NOMASS_CG;
    p.precision = precision;
    int calc_ssint = 1, calc_steric = 1;
    // keys of features this engine leaves out: they must be 0 (or absent)
    static const char *must_be_zero[] = {"calc_es", "calc_kinetics", "calc_springs", "calc_preComp",
                                         "sticky_wall_xz", "calc_steric_rod", "calc_vdw_rod", "num_rods",
                                         "num_interfaces", "force_pbc"};
    // keys that only configure those features (or output we do not write): accepted and ignored
    static const char *ignored[] = {"kappa", "epsilon_0", "dielec_ext", "es_update", "es_h", "wall_x_1", "wall_x_2",
                                    "wall_y_1", "wall_y_2", "wall_z_1", "wall_z_2", "vdw_forcefield_params",
                                    "ssint_forcefield_params", "vdw_in_fname", "ssint_in_fname", "ljparams",
                                    "lj_params", "ssint_type", "vdw_type", "steric_factor", "steric_dr",
                                    "num_states", "inc_self_ssint", "inc_self_vdw", "kinetics_update",
                                    "det_measurement_out_fname", "kinetics_out_fname", "beads_out_fname",
                                    "bsite_in_fname", "vdw_steric_factor", "vdw_steric_dr", "rod_lj_in_fname",
                                    "ssint_steric_dr"};
    for (const auto &ln : lines) {
        std::string k, v;
        parse_tag(ln, k, v);
        if (k == "param" || k == "/param") continue;
        bool done = true;
        if (k == "restart") restart = atoi(v.c_str());
        else if (k == "num_steps") num_steps = (long long)atof(v.c_str());
        else if (k == "check") check = (int)atof(v.c_str());
        else if (k == "rng_seed") { rng_seed = atoll(v.c_str()); seed_set = v != "time"; }
        else if (k == "trajectory_out_fname") traj_fname = join_dir(dir, v);
        else if (k == "measurement_out_fname") meas_fname = join_dir(dir, v);
        else if (k == "checkpoint_out") ockpt_fname = join_dir(dir, v);
        else if (k == "checkpoint_in") ickpt_fname = join_dir(dir, v);
        else if (k == "move_into_box") move_into_box = atoi(v.c_str());
        else if (k == "ssint_cutoff" || k == "vdw_cutoff") ssint_cutoff = atof(v.c_str()) / M_LENGTH;
        else if (k == "es_N_x") es_N[0] = atoi(v.c_str());
        else if (k == "es_N_y") es_N[1] = atoi(v.c_str());
        else if (k == "es_N_z") es_N[2] = atoi(v.c_str());
        else if (k == "calc_ssint" || k == "calc_vdw") calc_ssint = atoi(v.c_str());
        else if (k == "calc_steric") calc_steric = atoi(v.c_str());
        else if (k == "calc_ctforces") {
            calc_ctforces = atoi(v.c_str());
            if (calc_ctforces != 0 && calc_ctforces != 1) return fail("'calc_ctforces' must be 0 or 1");
        }
        else if (k == "num_blobs" || k == "num_conformations") {
            for (double x : tuple_values(v))
                if (k == "num_conformations" && x != 1.0) return fail("several conformations per blob are outside this engine");
        } else done = false;
        if (done) continue;
        if (std::find_if(std::begin(must_be_zero), std::end(must_be_zero), [&](const char *z) { return k == z; }) !=
            std::end(must_be_zero)) {
            if (atof(v.c_str()) != 0.0) return fail("'" + k + "' enables a feature outside this engine");
            continue;
        }
        if (std::find_if(std::begin(ignored), std::end(ignored), [&](const char *z) { return k == z; }) !=
            std::end(ignored))
            continue;
        // the hot-path keys: dt, kT, epsilon, max_iterations_cg, calc_noise, calc_stokes/do_stokes, stokes_visc
        if (ffea_gpu_params_assign(&p, k.c_str(), v.c_str()) != FFEA_GPU_OK)
            return fail("unsupported <param> key '" + k + "'");
    }
    if (calc_ssint != 0 || calc_steric != 0)
        return fail("surface-surface and steric interactions are outside this engine: set calc_ssint = 0 and "
                    "calc_steric = 0");
    if (check <= 0) return fail("check must be positive");
    const std::string base = script.substr(0, script.rfind('.') == std::string::npos ? script.size() : script.rfind('.'));
    if (traj_fname.empty()) traj_fname = base + ".ftj";
    if (meas_fname.empty()) meas_fname = base + ".fm";
    if (ockpt_fname.empty()) ockpt_fname = base + ".fcp";
    if (restart && ickpt_fname.empty()) return fail("restart needs checkpoint_in");
    if (!ickpt_fname.empty() && ickpt_fname == ockpt_fname) return fail("checkpoint_in and checkpoint_out must differ");
    return FFEA_GPU_OK;
}

// read_and_build_system's reading of <system> (src/World.cpp:2300-2700), one conformation per blob
int ffea_gpu_world::read_system(const std::vector<std::string> &lines) {
    int depth_blob = 0, depth_conf = 0, depth_inter = 0, depth_ctf = 0, ctf_fields = 0;
    BlobSpec cur;
    for (const auto &ln : lines) {
        std::string k, v;
        parse_tag(ln, k, v);
        if (k == "system" || k == "/system") continue;
        // <interactions>: only its <ctforces> block is read, and only with calc_ctforces = 1 (the blocks of
        // springs and pre-computed potentials belong to features that must be off)
        if (!depth_blob && k == "interactions") { depth_inter = 1; continue; }
        if (!depth_blob && k == "/interactions") { depth_inter = 0; continue; }
        if (depth_inter) {
            if (k == "ctforces") depth_ctf = 1;
            else if (k == "/ctforces") depth_ctf = 0;
            else if (depth_ctf && calc_ctforces) {
                ++ctf_fields;
                if (k != "ctforces_fname") return fail("ctforces_fname not provided in <ctforces> block");
                ctforces_fname = join_dir(dir, v);
            }
            continue;
        }
        if (k == "blob") { depth_blob = 1; cur = BlobSpec(); continue; }
        if (k == "/blob") {
            if (cur.scale <= 0) return fail("blob " + std::to_string(spec.size()) + ": scale not set");
            if (cur.motion_state != "DYNAMIC") return fail("only DYNAMIC blobs are supported");
            spec.push_back(cur);
            depth_blob = 0;
            continue;
        }
        if (k == "conformation") { depth_conf = 1; continue; }
        if (k == "/conformation") { depth_conf = 0; continue; }
        if (!depth_blob) return fail("<" + k + "> outside a blob block is outside this engine");
        if (depth_conf) {
            if (k == "nodes") cur.nodes = join_dir(dir, v);
            else if (k == "topology") cur.topology = join_dir(dir, v);
            else if (k == "material") cur.material = join_dir(dir, v);
            else if (k == "stokes") cur.stokes = join_dir(dir, v);
            else if (k == "pin") cur.pin = join_dir(dir, v);
            else if (k == "motion_state") cur.motion_state = v;
            else if (k == "surface") cur.surface = join_dir(dir, v);
            else if (k == "vdw" || k == "ssint" || k == "beads" || k == "binding_sites") continue;
            else return fail("unsupported conformation key '" + k + "'");
            continue;
        }
        if (k == "solver") {
            if (v == "CG_nomass") cur.solver = FFEA_GPU_NOMASS_CG;
            else if (v == "CG") cur.solver = FFEA_GPU_CG;
            else if (v == "masslumped") cur.solver = FFEA_GPU_MASSLUMPED;
            else return fail("unsupported solver '" + v + "'");
        } else if (k == "scale") {
            cur.scale = atof(v.c_str());
        } else if (k == "centroid" || k == "centroid_pos") {
            const auto t = tuple_values(v);
            if (t.size() != 3) return fail("centroid needs 3 values");
            cur.set_centroid = true;
            for (int c = 0; c < 3; ++c) cur.centroid[c] = t[c];
        } else if (k == "velocity") {
            const auto t = tuple_values(v);
            if (t.size() != 3) return fail("velocity needs 3 values");
            cur.set_velocity = true;
            for (int c = 0; c < 3; ++c) cur.velocity[c] = t[c] / M_VELOCITY;
        } else if (k == "rotation") {
            const auto t = tuple_values(v);
            if (t.size() != 3 && t.size() != 9) return fail("rotation needs 3 angles or 9 matrix entries");
            cur.rotation_type = t.size() == 3 ? 0 : 1;
            for (size_t i = 0; i < t.size(); ++i) cur.rotation[i] = t[i];
        } else if (k == "calc_compress" || k == "compress") {
            if (atof(v.c_str()) != 0.0 && k == "calc_compress") return fail("blob compression is outside this engine");
        } else {
            return fail("unsupported blob key '" + k + "'");
        }
    }
    if (spec.empty()) return fail("no <blob> in <system>");
    if (calc_ctforces) {
        if (ctf_fields != 1) return fail("only a single field is allowed in the <ctforces> block");
        std::ifstream probe(ctforces_fname);
        if (!probe) return fail("ctforces_fname: " + ctforces_fname + " could not be opened");
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_world::build() {
    const int nb = (int)spec.size();
    std::vector<std::vector<double>> pos(nb), vel(nb);
    for (int i = 0; i < nb; ++i) {
        const BlobSpec &s = spec[i];
        ffea_gpu_params bp = p;
        bp.solver = s.solver;
        if (s.solver != FFEA_GPU_NOMASS_CG) mass_in_system = true;
        ffea_gpu_blob *b = nullptr;
        int rc = ffea_gpu_blob_load(s.nodes.c_str(), s.topology.c_str(), s.material.c_str(),
                                    s.stokes.empty() ? nullptr : s.stokes.c_str(),
                                    s.pin.empty() ? nullptr : s.pin.c_str(), s.scale, &bp, &b);
        if (rc) return rc;
        blobs.push_back(b);
        n_all.push_back(b->h.n_all);
        if (calc_ctforces &&
            (rc = b->load_ctforces(ctforces_fname.c_str(), s.surface.empty() ? nullptr : s.surface.c_str(), i)))
            return rc;
        pos[i].resize(3 * (size_t)b->h.n_all);
        vel[i].assign(3 * (size_t)b->h.n_all, 0.0);
        if ((rc = ffea_gpu_blob_get_state(b, pos[i].data(), nullptr, nullptr))) return rc;
        auto centroid = [&](double c[3]) {
            c[0] = c[1] = c[2] = 0.0;
            for (int n = 0; n < b->h.n_all; ++n)
                for (int d = 0; d < 3; ++d) c[d] += pos[i][3 * (size_t)n + d];
            for (int d = 0; d < 3; ++d) c[d] *= 1.0 / b->h.n_all;
        };
        // Blob::position: the centroid moves to the given point (file units x scale)
        if (s.set_centroid) {
            double c[3];
            centroid(c);
            for (int n = 0; n < b->h.n_all; ++n)
                for (int d = 0; d < 3; ++d) pos[i][3 * (size_t)n + d] += s.centroid[d] * s.scale / M_LENGTH - c[d];
        }
        // Blob::rotate (src/Blob.cpp:538-600): about the centroid, by x, y, z angles in degrees or a matrix
        if (s.rotation_type >= 0) {
            double r[9];
            if (s.rotation_type == 0) {
                const double xa = s.rotation[0] * PI / 180.0, ya = s.rotation[1] * PI / 180.0,
                             za = s.rotation[2] * PI / 180.0;
                r[0] = cos(ya) * cos(za);
                r[1] = sin(xa) * sin(ya) * cos(za) - cos(xa) * sin(za);
                r[2] = cos(xa) * sin(ya) * cos(za) + sin(xa) * sin(za);
                r[3] = cos(ya) * sin(za);
                r[4] = sin(xa) * sin(ya) * sin(za) + cos(xa) * cos(za);
                r[5] = cos(xa) * sin(ya) * sin(za) - sin(xa) * cos(za);
                r[6] = -1 * sin(ya);
                r[7] = sin(xa) * cos(ya);
                r[8] = cos(xa) * cos(ya);
            } else {
                for (int k = 0; k < 9; ++k) r[k] = s.rotation[k];
            }
            double c[3];
            centroid(c);
            for (int n = 0; n < b->h.n_all; ++n) {
                double *q = &pos[i][3 * (size_t)n];
                const double x = q[0] - c[0], y = q[1] - c[1], z = q[2] - c[2];
                q[0] = x * r[0] + y * r[1] + z * r[2] + c[0];
                q[1] = x * r[3] + y * r[4] + z * r[5] + c[1];
                q[2] = x * r[6] + y * r[7] + z * r[8] + c[2];
            }
        }
        if (s.set_velocity)
            for (int n = 0; n < b->h.n_all; ++n)
                for (int d = 0; d < 3; ++d) vel[i][3 * (size_t)n + d] = s.velocity[d];
    }
    // World::init: the system's centroid goes to the centre of a box of ssint_cutoff x es_N cells
    // (es_N from the system's extent when unset, src/World.cpp:440-475)
    if (move_into_box == 1) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, wc[3] = {0, 0, 0};
        long long tot = 0;
        for (int i = 0; i < nb; ++i) {
            for (int n = 0; n < n_all[i]; ++n)
                for (int d = 0; d < 3; ++d) {
                    const double x = pos[i][3 * (size_t)n + d];
                    lo[d] = std::min(lo[d], x);
                    hi[d] = std::max(hi[d], x);
                    wc[d] += x;
                }
            tot += n_all[i];
        }
        double shift[3];
        for (int d = 0; d < 3; ++d) {
            int n = es_N[d];
            if (es_N[0] < 1 || es_N[1] < 1 || es_N[2] < 1) n = 2 * (int)ceil((hi[d] - lo[d]) / ssint_cutoff);
            shift[d] = ssint_cutoff * n / 2.0 - wc[d] / tot;
        }
        for (int i = 0; i < nb; ++i)
            for (int n = 0; n < n_all[i]; ++n)
                for (int d = 0; d < 3; ++d) pos[i][3 * (size_t)n + d] += shift[d];
    }
    for (int i = 0; i < nb; ++i) {
        int rc = ffea_gpu_blob_set_state(blobs[i], pos[i].data(), vel[i].data());
        if (!rc) rc = ffea_gpu_blob_set_rmsd_reference(blobs[i]);  // Blob::set_pos_0 after the moves
        if (rc) return rc;
    }
    // one stream for the World: blob i's elements start after blobs < i, its Stokes draws after every
    // element and after the Stokes draws of blobs < i
    unsigned long long elem_total = 0, stokes_total = 0;
    for (auto *b : blobs) {
        elem_total += b->element_draws();
        stokes_total += b->stokes_draws();
    }
    unsigned long long elem_before = 0, stokes_before = 0;
    for (auto *b : blobs) {
        int rc = b->set_rng_layout(elem_total + stokes_total, elem_total - elem_before + stokes_before);
        if (rc) return rc;
        elem_before += b->element_draws();
        stokes_before += b->stokes_draws();
    }
    // RngStream package seed from rng_seed (src/World.cpp:270-280): six (rand() + rand()) modulo m1, m2
    if (!restart) {
        srand((unsigned)(seed_set ? rng_seed : (long long)time(nullptr)));
        const uint32_t two_max[2] = {4294967087u, 4294944443u};
        for (int k = 0; k < 6; ++k) {
            const uint32_t a = (uint32_t)rand(), c = (uint32_t)rand();
            stream[k] = (uint32_t)((a + c) % two_max[k / 3]);
        }
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_world::open_outputs() {
    if (restart) {
        if (!(traj = fopen(traj_fname.c_str(), "ab"))) return fail("cannot open " + traj_fname);
        if (!(meas = fopen(meas_fname.c_str(), "ab"))) return fail("cannot open " + meas_fname);
        return FFEA_GPU_OK;
    }
    if (!(traj = fopen(traj_fname.c_str(), "wb"))) return fail("cannot open " + traj_fname);
    fprintf(traj, "FFEA_trajectory_file\n\nInitialisation:\nNumber of Blobs %d\nNumber of Conformations",
            (int)blobs.size());
    for (size_t i = 0; i < blobs.size(); ++i) fprintf(traj, " %d", 1);
    fprintf(traj, "\n");
    for (size_t i = 0; i < blobs.size(); ++i) fprintf(traj, "Blob %d:\tConformation %d Nodes %d\t\n", (int)i, 0, n_all[i]);
    fprintf(traj, "\n*\n");
    if (!(meas = fopen(meas_fname.c_str(), "wb"))) return fail("cannot open " + meas_fname);
    const time_t now = time(nullptr);
    const tm *lt = localtime(&now);
    fprintf(meas, "FFEA Global Measurement File\n\nSimulation Details:\n");
    fprintf(meas, "\tGB300 blob-step engine (ffea_gpu), %s precision\n", precision == FFEA_GPU_MIXED ? "mixed" : "FP64");
    fprintf(meas, "\tSimulation Began on %d/%d/%d at %d:%d:%d\n", lt->tm_mday, 1 + lt->tm_mon, 1900 + lt->tm_year,
            lt->tm_hour, lt->tm_min, lt->tm_sec);
    fprintf(meas, "\tScript Filename = %s\n", script.c_str());
    fprintf(meas, "\tSimulation Type = %s\n\n", "Full");
    fprintf(meas, "Parameters:\n\tSystem parameters:\n");
    fprintf(meas, "\trestart = %d\n\tdt = %e\n\tnum_steps = %lld\n\tcheck = %d\n\trng_seed = %lld\n", restart,
            p.dt * M_TIME, num_steps, check, rng_seed);
    fprintf(meas, "\tkT = %e\n\tmax_iterations_cg = %d\n\tepsilon = %e\n", p.kT * M_ENERGY, p.max_iterations_cg,
            sqrt(p.epsilon2));
    fprintf(meas, "\tnum_blobs = %d\n\tcalc_noise = %d\n\tcalc_stokes = %d\n\n", (int)blobs.size(), p.calc_noise,
            p.calc_stokes);
    fprintf(meas, "Measurements:\n%-14s", "Time");
    if (mass_in_system) fprintf(meas, "%-14s", "KineticEnergy");
    fprintf(meas, "%-14s", "StrainEnergy");
    fprintf(meas, "%-14s%-14s%-14s%-14s\n", "Centroid[0]", "Centroid[1]", "Centroid[2]", "RMSD");
    fflush(meas);
    return FFEA_GPU_OK;
}

// restart = 1: the stream from the checkpoint's first state line, positions (and velocities) from the
// trajectory's last complete frame, which is cut off (with its measurement line) to be written again
int ffea_gpu_world::restart_state() {
    {
        std::ifstream f(ickpt_fname);
        if (!f) return fail("cannot open " + ickpt_fname);
        std::string header, line;
        std::getline(f, header);
        if (!std::getline(f, line)) return fail("no RNG state in " + ickpt_fname);
        std::istringstream is(line);
        unsigned long long v[6];
        for (auto &x : v)
            if (!(is >> x)) return fail("malformed RNG state in " + ickpt_fname);
        for (int k = 0; k < 6; ++k) stream[k] = (uint32_t)v[k];
    }
    std::ifstream f(traj_fname, std::ios::binary);
    if (!f) return fail("cannot open " + traj_fname);
    std::string all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    // frames: "Blob 0, Conformation 0, step S\n" ... "*\nConformation Changes:\n" ... "*\n"
    const std::string head = "Blob 0, Conformation ";
    size_t last = std::string::npos, pos = 0;
    while ((pos = all.find(head, pos)) != std::string::npos) {
        if (pos == 0 || all[pos - 1] == '\n') {
            const size_t end = all.find("*\nConformation Changes:\n", pos);
            if (end != std::string::npos && all.find("*\n", end + 2) != std::string::npos) last = pos;
        }
        pos += head.size();
    }
    if (last == std::string::npos) return fail("no complete frame in " + traj_fname);
    std::istringstream is(all.substr(last));
    for (size_t b = 0; b < blobs.size(); ++b) {
        std::string line;
        std::getline(is, line);
        int bi = -1, ci = -1;
        long long st = -1;
        if (sscanf(line.c_str(), "Blob %d, Conformation %d, step %lld", &bi, &ci, &st) != 3 || bi != (int)b)
            return fail("unexpected frame header in " + traj_fname);
        step_initial = st;
        std::getline(is, line);  // DYNAMIC
        std::vector<double> P(3 * (size_t)n_all[b]), V(3 * (size_t)n_all[b]);
        for (int n = 0; n < n_all[b]; ++n) {
            double q[10];
            for (double &x : q)
                if (!(is >> x)) return fail("truncated frame in " + traj_fname);
            for (int d = 0; d < 3; ++d) {
                P[3 * (size_t)n + d] = q[d] / M_LENGTH;
                V[3 * (size_t)n + d] = q[3 + d] / M_VELOCITY;
            }
        }
        std::getline(is, line);
        int rc = ffea_gpu_blob_set_state(blobs[b], P.data(), spec[b].solver == FFEA_GPU_NOMASS_CG ? nullptr : V.data());
        if (rc) return rc;
    }
    // cut the trajectory before that frame and the measurement file before its last line
    {
        std::ofstream o(traj_fname, std::ios::binary | std::ios::trunc);
        o << all.substr(0, last);
    }
    std::ifstream fm(meas_fname, std::ios::binary);
    if (!fm) return fail("cannot open " + meas_fname);
    std::string m((std::istreambuf_iterator<char>(fm)), std::istreambuf_iterator<char>());
    fm.close();
    if (!m.empty() && m.back() == '\n') m.pop_back();
    const size_t nl = m.rfind('\n');
    m = m.substr(0, nl == std::string::npos ? 0 : nl + 1);
    std::ofstream om(meas_fname, std::ios::binary | std::ios::trunc);
    om << m;
    return FFEA_GPU_OK;
}

int ffea_gpu_world::write_checkpoint() {
    FILE *f = fopen(ockpt_fname.c_str(), "wb");
    if (!f) return fail("cannot open " + ockpt_fname);
    fprintf(f, "RNGStreams dedicated to the thermal stress: %d\n", 1);
    fprintf(f, "%u %u %u %u %u %u\n", stream[0], stream[1], stream[2], stream[3], stream[4], stream[5]);
    fclose(f);
    return FFEA_GPU_OK;
}

int ffea_gpu_world::write_frame(long long step) {
    for (size_t b = 0; b < blobs.size(); ++b) {
        fprintf(traj, "Blob %d, Conformation %d, step %lld\n", (int)b, 0, step);
        fprintf(traj, "DYNAMIC\n");
        std::vector<double> P(3 * (size_t)n_all[b]), V(3 * (size_t)n_all[b]);
        const bool nomass = spec[b].solver == FFEA_GPU_NOMASS_CG;
        int rc = ffea_gpu_blob_get_state(blobs[b], P.data(), nomass ? nullptr : V.data(), nullptr);
        if (rc) return rc;
        for (int n = 0; n < n_all[b]; ++n) {
            const double *q = &P[3 * (size_t)n];
            if (nomass)
                fprintf(traj, "%e %e %e %e %e %e %e %e %e %e\n", q[0] * M_LENGTH, q[1] * M_LENGTH, q[2] * M_LENGTH, 0.,
                        0., 0., 0., 0., 0., 0.);
            else {
                const double *v = &V[3 * (size_t)n];
                fprintf(traj, "%e %e %e %e %e %e %e %e %e %e\n", q[0] * M_LENGTH, q[1] * M_LENGTH, q[2] * M_LENGTH,
                        v[0] * M_VELOCITY, v[1] * M_VELOCITY, v[2] * M_VELOCITY, 0., 0., 0., 0.);
            }
        }
    }
    fprintf(traj, "*\nConformation Changes:\n");
    for (size_t b = 0; b < blobs.size(); ++b) fprintf(traj, "Blob %d: Conformation %d -> Conformation %d\n", (int)b, 0, 0);
    fprintf(traj, "*\n");
    fflush(traj);
    return FFEA_GPU_OK;
}

int ffea_gpu_world::write_measurement(long long step) {
    double ke = 0, se = 0, cog[3] = {0, 0, 0}, r2 = 0;
    long long tot = 0;
    for (size_t b = 0; b < blobs.size(); ++b) {
        double o[6];
        int rc = ffea_gpu_blob_measurements(blobs[b], o);
        if (rc) return rc;
        se += o[0];
        ke += o[1];
        for (int d = 0; d < 3; ++d) cog[d] += o[2 + d] * n_all[b];
        r2 += o[5] * o[5] * n_all[b];
        tot += n_all[b];
    }
    fprintf(meas, "%-14.6e", step * p.dt * M_TIME);
    if (mass_in_system) fprintf(meas, "%-14.6e", ke * M_ENERGY);
    fprintf(meas, "%-14.6e", se * M_ENERGY);
    fprintf(meas, "%-14.6e%-14.6e%-14.6e", cog[0] / tot * M_LENGTH, cog[1] / tot * M_LENGTH, cog[2] / tot * M_LENGTH);
    fprintf(meas, "%-14.6e\n", sqrt(r2 / tot) * M_LENGTH);
    fflush(meas);
    return FFEA_GPU_OK;
}

// World::run (src/World.cpp:1747-2059): for step = step_initial .. num_steps, checkpoint before the forces and
// trajectory + measurements after them every `check` steps, then the update. Between outputs the blobs step
// `check` steps at a time (their streams advance by the World's draws on the device).
int ffea_gpu_world::run(long long *last_step) {
    unsigned long long elem_before = 0, total = 0;
    for (auto *b : blobs) total += b->element_draws() + b->stokes_draws();
    const MrgJump step_jump = jump_pow(total);
    // each blob's stream: the World's stream past the elements of the blobs before it
    auto place_streams = [&]() -> int {
        elem_before = 0;
        for (auto *b : blobs) {
            uint32_t o[6];
            mrg_apply(jump_pow(elem_before), stream, o);
            int rc = ffea_gpu_blob_set_rng_state(b, o);
            if (rc) return rc;
            elem_before += b->element_draws();
        }
        return FFEA_GPU_OK;
    };
    long long step = step_initial;
    int rc0 = place_streams();
    if (rc0) return rc0;
    while (step <= num_steps) {
        if (step % check == 0) {
            int rc = write_checkpoint();
            if (!rc) rc = place_streams();
            if (rc) return rc;
            if ((rc = write_frame(step)) || (rc = write_measurement(step))) return rc;
        }
        const long long next = std::min(num_steps + 1, (step / check + 1) * check);
        const int n = (int)(next - step);
        for (auto *b : blobs) {
            int done = 0;
            int rc = ffea_gpu_blob_step(b, n, &done);
            if (rc) {
                if (last_step) *last_step = step + done;
                return rc;
            }
        }
        for (int k = 0; k < n; ++k) {
            uint32_t o[6];
            mrg_apply(step_jump, stream, o);
            std::copy(o, o + 6, stream);
        }
        step = next;
    }
    if (last_step) *last_step = num_steps;
    return FFEA_GPU_OK;
}

extern "C" {

int ffea_gpu_world_load(const char *script, int precision, ffea_gpu_world **out) {
    if (!script || !out || (precision != FFEA_GPU_FP64 && precision != FFEA_GPU_MIXED)) return FFEA_GPU_EINPUT;
    *out = nullptr;
    std::unique_ptr<ffea_gpu_world> w(new (std::nothrow) ffea_gpu_world());
    if (!w) return FFEA_GPU_ENOMEM;
    w->precision = precision;
    w->script = script;
    const size_t sl = w->script.rfind('/');
    w->dir = sl == std::string::npos ? "" : w->script.substr(0, sl);
    std::vector<std::string> lines;
    if (!script_lines(script, lines)) {
        g_last_error = std::string("cannot read ") + script;
        return FFEA_GPU_EFILE;
    }
    // FFEA_input_reader::extract_block for <param> and <system>
    auto block = [&](const std::string &name, std::vector<std::string> &outb) {
        bool in = false;
        for (const auto &l : lines) {
            std::string k, v;
            parse_tag(l, k, v);
            if (k == name) { in = true; continue; }
            if (k == "/" + name) { in = false; continue; }
            if (in) outb.push_back(l);
        }
    };
    std::vector<std::string> params, system;
    block("param", params);
    block("system", system);
    int rc = w->read_params(params);
    if (!rc) rc = w->read_system(system);
    if (!rc) rc = w->build();
    if (!rc && w->restart) rc = w->restart_state();
    if (!rc) rc = w->open_outputs();
    if (rc) return rc;
    *out = w.release();
    return FFEA_GPU_OK;
}

int ffea_gpu_world_run(ffea_gpu_world *w, long long *last_step) {
    if (!w) return FFEA_GPU_EINPUT;
    return w->run(last_step);
}

int ffea_gpu_world_num_blobs(ffea_gpu_world *w) { return w ? (int)w->blobs.size() : 0; }

ffea_gpu_blob *ffea_gpu_world_blob(ffea_gpu_world *w, int i) {
    if (!w || i < 0 || i >= (int)w->blobs.size()) return nullptr;
    return w->blobs[i];
}

void ffea_gpu_world_destroy(ffea_gpu_world *w) { delete w; }

}  // extern "C"
