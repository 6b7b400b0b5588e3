// io.cu -- the reference's input formats for the hot path.
//
//  * ffea_gpu_params_assign: SimulationParams::assign for the hot-path keys
//    of a .ffea <param> block (src/SimulationParams.cpp:245-560).
//  * ffea_gpu_blob_load: Blob::load_nodes / load_topology /
//    load_material_params / load_stokes_params / load_pinned_nodes
//    (src/Blob.cpp:1911-2083, 2241-2353, 3024-3076) followed by
//    ffea_gpu_blob_create; same header lines, same checks, same unit
//    conversion (positions and Stokes radii times scale/mesoDimensions::length,
//    src/World.cpp:2632).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"

namespace {

constexpr double MESO_LENGTH = 1.7e-10;
constexpr double MESO_ENERGY = 4.141945559999999e-21;
constexpr double MESO_TIME = 3.7302915560886126e-13;
constexpr double MESO_PRESSURE = 8.4305832688784826e8;

struct File {
    FILE *f = nullptr;
    explicit File(const char *path) : f(path ? fopen(path, "r") : nullptr) {}
    ~File() {
        if (f) fclose(f);
    }
};

bool header(FILE *f, const char *kind) {
    char line[64];
    if (!fgets(line, sizeof line, f)) return false;
    std::string a = std::string("ffea ") + kind + "\n", b = std::string("walrus ") + kind + "\n";
    return a == line || b == line;
}

bool line_is(FILE *f, const char *want) {
    char line[64];
    if (!fgets(line, sizeof line, f)) return false;
    return std::strcmp(line, want) == 0;
}

}  // namespace

extern "C" {

int ffea_gpu_params_assign(ffea_gpu_params *p, const char *key, const char *value) {
    if (!p || !key || !value) return FFEA_GPU_EINPUT;
    const std::string k(key);
    if (k == "dt") {
        p->dt = atof(value);
        p->dt /= MESO_TIME;
    } else if (k == "kT") {
        p->kT = atof(value);
        p->kT /= MESO_ENERGY;
    } else if (k == "epsilon") {
        p->epsilon2 = atof(value);
        p->epsilon2 *= p->epsilon2;
    } else if (k == "max_iterations_cg") {
        p->max_iterations_cg = atoi(value);
    } else if (k == "calc_noise") {
        p->calc_noise = atoi(value);
    } else if (k == "calc_stokes" || k == "do_stokes") {
        p->calc_stokes = atoi(value);
    } else if (k == "stokes_visc") {
        p->stokes_visc = atof(value);
        p->stokes_visc /= MESO_PRESSURE * MESO_TIME;
    } else if (k == "solver") {
        const std::string v(value);
        if (v == "CG_nomass") p->solver = FFEA_GPU_NOMASS_CG;
        else if (v == "CG") p->solver = FFEA_GPU_CG;
        else if (v == "masslumped") p->solver = FFEA_GPU_MASSLUMPED;
        else return FFEA_GPU_EINPUT;
    } else if (k == "precision") {
        const std::string v(value);
        if (v == "fp64") p->precision = FFEA_GPU_FP64;
        else if (v == "mixed") p->precision = FFEA_GPU_MIXED;
        else return FFEA_GPU_EINPUT;
    } else if (k == "cg_poly") {
        const int v = atoi(value);
        if (v < -1 || v > FFEA_GPU_CG_POLY_MAX || (v > 0 && v % 2 != 0)) return FFEA_GPU_EINPUT;
        p->cg_poly = v;
    } else if (k == "cg_smem_blocks") {
        const int v = atoi(value);
        if (v < -1) return FFEA_GPU_EINPUT;
        p->cg_smem_blocks = v;
    } else {
        return FFEA_GPU_EINPUT;
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_blob_load(const char *node_file, const char *top_file, const char *mat_file, const char *stokes_file,
                       const char *pin_file, double scale, const ffea_gpu_params *params, ffea_gpu_blob **out) {
    if (!out || !params) return FFEA_GPU_EINPUT;
    *out = nullptr;
    const double s = scale / MESO_LENGTH;
    // nodes
    File fn(node_file);
    if (!fn.f || !header(fn.f, "node file")) return FFEA_GPU_EFILE;
    int num_nodes = 0, num_surf = 0, num_int = 0;
    if (fscanf(fn.f, "num_nodes %d\n", &num_nodes) != 1 || fscanf(fn.f, "num_surface_nodes %d\n", &num_surf) != 1 ||
        fscanf(fn.f, "num_interior_nodes %d\n", &num_int) != 1 || num_nodes <= 0)
        return FFEA_GPU_EFILE;
    if (!line_is(fn.f, "surface nodes:\n")) return FFEA_GPU_EFILE;
    std::vector<double> pos(3 * (size_t)num_nodes);
    for (int i = 0; i < num_nodes; ++i) {
        if (i == num_surf && !line_is(fn.f, "interior nodes:\n")) return FFEA_GPU_EFILE;
        double x, y, z;
        if (fscanf(fn.f, "%le %le %le\n", &x, &y, &z) != 3) return FFEA_GPU_EFILE;
        pos[3 * (size_t)i] = s * x;
        pos[3 * (size_t)i + 1] = s * y;
        pos[3 * (size_t)i + 2] = s * z;
    }
    // topology
    File ft(top_file);
    if (!ft.f || !header(ft.f, "topology file")) return FFEA_GPU_EFILE;
    int ne = 0, nse = 0, nie = 0;
    if (fscanf(ft.f, "num_elements %d\n", &ne) != 1 || fscanf(ft.f, "num_surface_elements %d\n", &nse) != 1 ||
        fscanf(ft.f, "num_interior_elements %d\n", &nie) != 1 || ne <= 0)
        return FFEA_GPU_EFILE;
    if (!line_is(ft.f, "surface elements:\n")) return FFEA_GPU_EFILE;
    std::vector<int> tets(10 * (size_t)ne);
    for (int e = 0; e < ne; ++e) {
        if (e == nse && !line_is(ft.f, "interior elements:\n")) return FFEA_GPU_EFILE;
        int *t = &tets[10 * (size_t)e];
        if (fscanf(ft.f, "%d %d %d %d %d %d %d %d %d %d\n", t, t + 1, t + 2, t + 3, t + 4, t + 5, t + 6, t + 7,
                   t + 8, t + 9) != 10)
            return FFEA_GPU_EFILE;
        for (int j = 0; j < 10; ++j)
            if (t[j] < 0 || t[j] >= num_nodes) return FFEA_GPU_EINPUT;
    }
    // material
    File fm(mat_file);
    if (!fm.f || !header(fm.f, "material params file")) return FFEA_GPU_EFILE;
    int nm = 0;
    if (fscanf(fm.f, "num_elements %d\n", &nm) != 1 || nm != ne) return FFEA_GPU_EFILE;
    std::vector<double> mat6(6 * (size_t)ne);
    for (int e = 0; e < ne; ++e) {
        double *m = &mat6[6 * (size_t)e];
        if (fscanf(fm.f, "%le %le %le %le %le %le\n", m, m + 1, m + 2, m + 3, m + 4, m + 5) != 6) return FFEA_GPU_EFILE;
    }
    std::vector<double> rho(ne), A(ne), B(ne), G(ne), E(ne);
    ffea_gpu_material_from_si(ne, mat6.data(), rho.data(), A.data(), B.data(), G.data(), E.data());
    // stokes radii
    std::vector<double> radius(num_nodes, 0.0);
    if (stokes_file) {
        File fs(stokes_file);
        if (!fs.f || !header(fs.f, "stokes radii file")) return FFEA_GPU_EFILE;
        int ns = 0;
        if (fscanf(fs.f, "num_nodes %d\n", &ns) != 1 || ns != num_nodes) return FFEA_GPU_EFILE;
        for (int i = 0; i < num_nodes; ++i) {
            double r;
            if (fscanf(fs.f, "%le\n", &r) != 1) return FFEA_GPU_EFILE;
            radius[i] = r * s;
        }
    } else if (params->calc_stokes == 1) {
        return FFEA_GPU_EFILE;
    }
    // pinned nodes
    std::vector<int> pinned;
    if (pin_file && pin_file[0]) {
        File fp(pin_file);
        if (!fp.f || !header(fp.f, "pinned nodes file")) return FFEA_GPU_EFILE;
        int np = 0;
        if (fscanf(fp.f, "num_pinned_nodes %d\n", &np) != 1 || np < 0) return FFEA_GPU_EFILE;
        if (!line_is(fp.f, "pinned nodes:\n")) return FFEA_GPU_EFILE;
        pinned.resize(np);
        for (int i = 0; i < np; ++i) {
            if (fscanf(fp.f, "%d\n", &pinned[i]) != 1) return FFEA_GPU_EFILE;
            if (pinned[i] < 0 || pinned[i] >= num_nodes) return FFEA_GPU_EINPUT;
        }
    }
    ffea_gpu_mesh m{};
    m.num_nodes = num_nodes;
    m.num_elements = ne;
    m.num_pinned = (int)pinned.size();
    m.pos = pos.data();
    m.tets = tets.data();
    m.rho = rho.data();
    m.A = A.data();
    m.B = B.data();
    m.G = G.data();
    m.E = E.data();
    m.stokes_radius = radius.data();
    m.pinned = pinned.empty() ? nullptr : pinned.data();
    return ffea_gpu_blob_create(&m, params, out);
}

}  // extern "C"
