// nf_api.cu -- the C ABI (include/nanofiller_gb300.h) over the GB300 engine,
// the reference keyword parser and the reference file formats.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "nf_engine.cuh"

namespace nf {
unsigned long long g_launches = 0;
unsigned long long g_allocs = 0;
}

struct nf_handle {
    nf::Engine E;
    nf_params p;
    int cur = 0;  // realisation the per-realisation getters report (nf_select)
};

namespace {

nf_status fail(nf_handle* h, nf_status s, const std::string& msg) {
    if (h) h->E.err = msg;
    return s;
}

// Calls that read or write one realisation's files, rods or statistics run on
// single-realisation handles (nf_create); a batch handle reports through
// nf_select + nf_get_rods / nf_get_contacts / nf_batch_results.
#define NF_SINGLE(h, what)                                                                          \
    do {                                                                                            \
        if ((h)->E.R != 1) return fail((h), NF_ERR_STATE, what " runs on a single-realisation handle"); \
    } while (0)

bool read_density(const char* path, int ext[3], float dim[3], std::vector<float>* vals) {
    // read_density (src/IO.cpp:11-36): "Lx Ly Lz" "nx ny nz" then nx*ny*nz values.
    std::ifstream f(path);
    if (!f.is_open()) return false;
    if (!(f >> dim[0] >> dim[1] >> dim[2] >> ext[0] >> ext[1] >> ext[2])) return false;
    if (ext[0] <= 0 || ext[1] <= 0 || ext[2] <= 0) return false;
    size_t n = (size_t)ext[0] * ext[1] * ext[2];
    if (vals) {
        vals->resize(n);
        for (size_t i = 0; i < n; ++i)
            if (!(f >> (*vals)[i])) return false;
    }
    return true;
}

nf_status validate(const nf_params& p, std::string* why) {
    for (int d = 0; d < 3; ++d)
        if (!(p.box[d] > 0)) { *why = "box edges must be positive"; return NF_ERR_PARAM; }
    if (!(p.l > 0) || !(p.a > 0)) { *why = "rod length and radius must be positive"; return NF_ERR_PARAM; }
    if (!(p.vf > 0) && p.n_target <= 0) { *why = "volume fraction or target count required"; return NF_ERR_PARAM; }
    if (p.field_dir != 0 && p.field_dir != 1 && p.field_dir != 2 && p.field_dir != 4) {
        *why = "FIELD_DIR must be 0, 1, 2 or 4"; return NF_ERR_PARAM;
    }
    if (p.solve_method < 0 || p.solve_method > 3) { *why = "SOLVE_METHOD must be 0, 1, 2 or 3"; return NF_ERR_PARAM; }
    if (p.self_align_step < 0 || p.clust_flag < 0 || p.clust_flag > 1 || p.reduce_flag < 0 || p.reduce_flag > 1) {
        *why = "SELF_ALLIGN_STEP must be >= 0, CLUST_FLAG and REDUCE_FLAG 0 or 1"; return NF_ERR_PARAM;
    }
    if (!(p.clust_dist >= 0) || !(p.clust_angl >= 0 && p.clust_angl <= 1.5707964f) || !(p.align_cell >= 0) ||
        p.align_min < 0 || p.epoch_candidates < 0) {
        *why = "CLUST_DIST_LIM >= 0, CLUST_ANGL_LIM in [0, pi/2], ALIGN_CELL >= 0, ALIGN_MIN_RODS >= 0 and "
               "EPOCH_CANDIDATES >= 0 required";
        return NF_ERR_PARAM;
    }
    if (p.clust_flag) {  // a candidate's neighbours are searched among the images -1..1
        const float lmax = p.len_mode == NF_SIZE_LOGNORMAL ? p.len_max : p.l;
        for (int d = 0; d < 3; ++d)
            if (p.box[d] < lmax) { *why = "clusterisation needs box edges of at least the longest rod"; return NF_ERR_PARAM; }
    }
    if ((p.theta_dev > 0 || p.phi_dev > 0) && p.orient_mode == NF_ORIENT_VMF) {
        *why = "ORIENT VMF and DEF_THETA_DEV / DEF_PHI_DEV > 0 are exclusive orientation laws"; return NF_ERR_PARAM;
    }
    if ((p.theta_dev > 0 || p.phi_dev > 0) && p.self_align_step > 0 && p.align_law == 0) {
        *why = "ALIGN_LAW 0 refits von Mises-Fisher laws; with DEF_THETA_DEV / DEF_PHI_DEV > 0 use ALIGN_LAW 1 "
               "(the reference's truncated-normal cell laws)";
        return NF_ERR_UNSUPPORTED;
    }
    if (!std::isfinite(p.theta_med) || !std::isfinite(p.phi_med) || !std::isfinite(p.theta_dev) ||
        !std::isfinite(p.phi_dev) || p.ref_trunc_normal < 0 || p.ref_trunc_normal > 1) {
        *why = "DEF_THETA_* / DEF_PHI_* must be finite and TRUNC_NORMAL_REF 0 or 1"; return NF_ERR_PARAM;
    }
    if (p.orient_mode == NF_ORIENT_VMF && !(p.vmf_kappa > 0)) { *why = "VMF_KAPPA must be positive"; return NF_ERR_PARAM; }
    if (p.len_mode == NF_SIZE_LOGNORMAL && !(p.len_min > 0 && p.len_max >= p.len_min)) {
        *why = "LEN_CLIP lo hi required for lognormal lengths"; return NF_ERR_PARAM;
    }
    if (p.rad_mode == NF_SIZE_UNIFORM && !(p.rad_min > 0 && p.rad_max >= p.rad_min)) {
        *why = "RAD_RANGE lo hi required for uniform radii"; return NF_ERR_PARAM;
    }
    if (!(p.lambda > 0) || !(p.G0 > 0)) { *why = "tunnelling law needs G0 > 0 and lambda > 0"; return NF_ERR_PARAM; }
    if (!std::isfinite(p.tube_load)) { *why = "TUBE_LOAD must be finite"; return NF_ERR_PARAM; }
    if (p.align_law < 0 || p.align_law > 1) { *why = "ALIGN_LAW must be 0 or 1"; return NF_ERR_PARAM; }
    if (p.autotune < 0 || p.autotune > 1) { *why = "AUTOTUNE must be 0 or 1"; return NF_ERR_PARAM; }
    if (p.stencil_radius < 0 || p.stencil_radius > 2 || !(p.round_overshoot >= 0) || p.two_phase_work != p.two_phase_work) {
        *why = "STENCIL_RADIUS must be 0, 1 or 2 and ROUND_OVERSHOOT >= 0"; return NF_ERR_PARAM;
    }
    if (!(p.rod_sigma > 0)) { *why = "ROD_CONDUCTIVITY must be positive"; return NF_ERR_PARAM; }
    if (p.elec_buffer != 0 && p.elec_buffer != 1) { *why = "ELEC_BUFFER must be 0 or 1"; return NF_ERR_PARAM; }
    double reach = nf::stage_reach(p);
    for (int d = 0; d < 3; ++d)
        if ((p.gen_periodic >> d & 1) && p.box[d] < reach) {
            *why = "a periodic box edge is shorter than the pair reach (rod would meet its own image)";
            return NF_ERR_PARAM;
        }
    return NF_OK;
}

float rad(float deg, float pi) { return deg / 180 * pi; }

}  // namespace

extern "C" {

int nf_abi_version(void) { return NF_ABI_VERSION; }

const char* nf_status_string(nf_status s) {
    switch (s) {
        case NF_OK: return "ok";
        case NF_ERR_PARAM: return "invalid parameter";
        case NF_ERR_CUDA: return "CUDA error";
        case NF_ERR_NO_DEVICE: return "no CUDA device";
        case NF_ERR_ALLOC: return "allocation failed";
        case NF_ERR_CAPACITY: return "buffer too small";
        case NF_ERR_OVERFLOW: return "internal list overflow";
        case NF_ERR_NOT_CONVERGED: return "solve not converged";
        case NF_ERR_IO: return "I/O error";
        case NF_ERR_FORMAT: return "malformed file";
        case NF_ERR_STATE: return "call out of order";
        case NF_ERR_UNSUPPORTED: return "unsupported option";
        case NF_ERR_TIMEOUT: return "bounded wait expired";
    }
    return "unknown status";
}

nf_status nf_params_default(nf_params* p) {
    if (!p) return NF_ERR_PARAM;
    std::memset(p, 0, sizeof(*p));
    // simPrms::simPrms (src/simPrms.cpp:22-117)
    p->vf = 0.05f / 100.0f;
    p->vf_precision = 0.05f;
    p->theta_med = 0; p->theta_dev = -1; p->phi_med = 0; p->phi_dev = -1;
    p->l = 4; p->a = 0.010f; p->l_dev = -1; p->a_dev = -1;
    p->tol = 1.e-6f;
    p->sep = 0; p->sc_frac = 1.0f;
    p->stat_dist_lim = 0.015f;
    p->wrt_bin = 0;
    p->self_align_step = 0;  // the reference defaults to 50 (and samples isotropically
                             // while DEF_THETA_DEV is -1); here adaptation is asked for
    p->clust_flag = 0; p->reduce_flag = 0;
    p->clust_dist = 0.015f;
    p->clust_angl = 3.14159265359f / 12;  // Pi/12, src/simPrms.cpp:62-63
    p->align_cell = 0;
    p->align_min = 4;
    p->epoch_candidates = 0;
    // project keys
    p->seed = 0;
    p->n_candidates = 1ull << 20;
    p->n_target = 0;
    p->gen_periodic = 7;
    p->field_dir = 4;
    p->orient_mode = NF_ORIENT_ISOTROPIC;
    p->density_default = 1.0f;
    p->G0 = 1e-5;
    p->lambda = 0.18e-3;
    p->d_c = 0.34e-3;
    p->screening = 1;
    p->solve_max_iter = 20000;
    p->rod_sigma = 67.0;  // 6.7e7 S/m (tools/kirchhoff/kirchhoff.py:68)
    p->solve_tol = 1e-10;
    return NF_OK;
}

nf_status nf_params_from_file(const char* path, nf_params* p, int* n_unknown) {
    if (!path || !p) return NF_ERR_PARAM;
    std::ifstream f(path);
    if (!f.is_open()) return NF_ERR_IO;
    const float PI_ = 3.141593f, Pi = 3.14159265359f;  // inc/vectorMath.h:7, inc/simPrms.h:82
    int unknown = 0;
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty()) continue;
        size_t k = line.find_first_of(" \t");
        std::string key = line.substr(0, k);
        std::string rest = k == std::string::npos ? "" : line.substr(k + 1);
        std::istringstream in(rest);
        if (key.empty() || key[0] == '#') continue;
        float v;
        if (key == "WRT_BIN") in >> p->wrt_bin;
        else if (key == "VOLUME_PERCENT") { in >> v; p->vf = v / 100; }
        else if (key == "VOLUME_PERCENT_LIST") { int n; in >> n; for (int i = 0; i < n; ++i) in >> v; }
        else if (key == "VOL_FRAC_PRECISION") in >> p->vf_precision;
        else if (key == "SPAT_DISTR_FILE") {
            std::string name;
            in >> name;
            if (name == "NONE") {
                in >> p->box[0] >> p->box[1] >> p->box[2] >> p->mesh_ext[0] >> p->mesh_ext[1] >> p->mesh_ext[2];
                p->density_file[0] = 0;
            } else {
                std::snprintf(p->density_file, sizeof(p->density_file), "%s", name.c_str());
            }
        }
        else if (key == "PREF_ORT_PHI") { in >> v; p->pref_ort[0] = rad(v, PI_); }
        else if (key == "PREF_ORT_THETA") { in >> v; p->pref_ort[1] = rad(v, Pi); }
        else if (key == "DEF_THETA_MED") { in >> v; p->theta_med = rad(v, Pi); }
        else if (key == "DEF_PHI_MED") { in >> v; p->phi_med = rad(v, Pi); }
        else if (key == "DEF_THETA_DEV") { in >> v; p->theta_dev = v > 0 ? rad(v, Pi) : -1; }
        else if (key == "DEF_PHI_DEV") { in >> v; p->phi_dev = v > 0 ? rad(v, Pi) : -1; }
        else if (key == "INC_LEN_MED") in >> p->l;
        else if (key == "INC_LEN_DEV") in >> p->l_dev;
        else if (key == "INC_RAD_MED") in >> p->a;
        else if (key == "INC_RAD_DEV") in >> p->a_dev;
        else if (key == "INC_SEPARATION") in >> p->sep;
        else if (key == "INC_SOFTCORE") in >> p->sc_frac;
        else if (key == "STAT_DIST_LIM") in >> p->stat_dist_lim;
        else if (key == "SELF_ALLIGN_STEP") in >> p->self_align_step;
        else if (key == "REDUCE_FLAG") in >> p->reduce_flag;
        else if (key == "CLUST_FLAG") in >> p->clust_flag;
        else if (key == "CLUST_DIST_LIM") in >> p->clust_dist;
        else if (key == "CLUST_ANGL_LIM") in >> p->clust_angl;  // radians, read as is (src/simPrms.cpp:307)
        else if (key == "ALIGN_CELL") in >> p->align_cell;
        else if (key == "ALIGN_MIN_RODS") in >> p->align_min;
        else if (key == "EPOCH_CANDIDATES") { long long s; in >> s; p->epoch_candidates = s; }
        else if (key == "SOLVE_METHOD") in >> p->solve_method;
        else if (key == "SPAT_DIMENSIONS" ||
                 key == "ORNT_DISTR_FILE" || key == "IDIM_DISTR_FILE" || key == "MATH_TOLERANCE" ||
                 key == "DMN_CELL_MARGE") { /* parsed and ignored, as the reference does */ }
        // project keys
        else if (key == "SEED") { unsigned long long s; in >> s; p->seed = s; }
        else if (key == "CANDIDATES") { unsigned long long s; in >> s; p->n_candidates = s; }
        else if (key == "TARGET_COUNT") { long long s; in >> s; p->n_target = s; }
        else if (key == "PERIODIC") in >> p->gen_periodic;
        else if (key == "FIELD_DIR") in >> p->field_dir;
        else if (key == "ORIENT") {
            std::string m; in >> m;
            p->orient_mode = (m == "VMF" || m == "1") ? NF_ORIENT_VMF : NF_ORIENT_ISOTROPIC;
        }
        else if (key == "VMF_KAPPA") in >> p->vmf_kappa;
        else if (key == "LEN_LAW") { std::string m; in >> m; p->len_mode = (m == "LOGNORMAL" || m == "1") ? NF_SIZE_LOGNORMAL : NF_SIZE_CONST; }
        else if (key == "LEN_SIGMA_LN") in >> p->len_sigma_ln;
        else if (key == "LEN_CLIP") in >> p->len_min >> p->len_max;
        else if (key == "RAD_LAW") { std::string m; in >> m; p->rad_mode = (m == "UNIFORM" || m == "2") ? NF_SIZE_UNIFORM : NF_SIZE_CONST; }
        else if (key == "RAD_RANGE") in >> p->rad_min >> p->rad_max;
        else if (key == "DENSITY_DEFAULT") in >> p->density_default;
        else if (key == "CELL_EDGE") in >> p->cell_edge;
        else if (key == "TUNNEL_G0") in >> p->G0;
        else if (key == "TUNNEL_LAMBDA") in >> p->lambda;
        else if (key == "TUNNEL_DC") in >> p->d_c;
        else if (key == "REF_PARALLEL_TYPO") in >> p->ref_parallel_typo;
        else if (key == "TRUNC_NORMAL_REF") in >> p->ref_trunc_normal;
        else if (key == "TUBE_LOAD") in >> p->tube_load;
        else if (key == "ALIGN_LAW") in >> p->align_law;
        else if (key == "AUTOTUNE") in >> p->autotune;
        else if (key == "SCREENING") in >> p->screening;
        else if (key == "ROUND_CANDIDATES") in >> p->round_candidates;
        else if (key == "SOLVE_MAX_ITER") in >> p->solve_max_iter;
        else if (key == "SOLVE_TOL") in >> p->solve_tol;
        else if (key == "STENCIL_RADIUS") in >> p->stencil_radius;
        else if (key == "ROUND_OVERSHOOT") in >> p->round_overshoot;
        else if (key == "TWO_PHASE_WORK") in >> p->two_phase_work;
        else if (key == "ROD_CONDUCTIVITY") in >> p->rod_sigma;
        else if (key == "ELEC_BUFFER") in >> p->elec_buffer;
        else ++unknown;  // the reference prints "UNRECOGNISED STRING FOUND" and continues
    }
    if (n_unknown) *n_unknown = unknown;
    return NF_OK;
}

nf_status nf_target_count(const nf_params* p, int64_t* n) {
    if (!p || !n) return NF_ERR_PARAM;
    *n = nf::target_count(*p);
    return NF_OK;
}

nf_status nf_read_density_file(const char* path, int ext[3], float dim[3], float* values, size_t capacity) {
    if (!path || !ext || !dim) return NF_ERR_PARAM;
    std::vector<float> v;
    std::ifstream f(path);
    if (!f.is_open()) return NF_ERR_IO;
    f.close();
    if (!read_density(path, ext, dim, values ? &v : nullptr)) return NF_ERR_FORMAT;
    if (values) {
        if (capacity < v.size()) return NF_ERR_CAPACITY;
        std::copy(v.begin(), v.end(), values);
    }
    return NF_OK;
}

nf_status nf_create(const nf_params* p, nf_handle** out) {
    if (!p || !out) return NF_ERR_PARAM;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NF_ERR_NO_DEVICE;
    nf_handle* h = new (std::nothrow) nf_handle();
    if (!h) return NF_ERR_ALLOC;
    h->p = *p;
    std::vector<float> mesh;
    if (h->p.density_file[0]) {
        int ext[3];
        float dim[3];
        std::ifstream f(h->p.density_file);
        if (!f.is_open()) { delete h; return NF_ERR_IO; }
        f.close();
        if (!read_density(h->p.density_file, ext, dim, &mesh)) { delete h; return NF_ERR_FORMAT; }
        for (int d = 0; d < 3; ++d) { h->p.box[d] = dim[d]; h->p.mesh_ext[d] = ext[d]; }
    }
    std::string why;
    nf_status s = validate(h->p, &why);
    if (s != NF_OK) { delete h; return s; }
    std::vector<const float*> meshes(1, mesh.empty() ? nullptr : mesh.data());
    if (mesh.empty()) h->p.mesh_ext[0] = h->p.mesh_ext[1] = h->p.mesh_ext[2] = 0;
    s = h->E.init(&h->p, 1, meshes);
    if (s != NF_OK) { delete h; return s; }
    *out = h;
    return NF_OK;
}

nf_status nf_destroy(nf_handle* h) {
    if (!h) return NF_ERR_PARAM;
    h->E.release();
    delete h;
    return NF_OK;
}

nf_status nf_set_stream(nf_handle* h, void* stream) {
    if (!h) return NF_ERR_PARAM;
    h->E.st = (cudaStream_t)stream;
    return NF_OK;
}

nf_status nf_last_error(const nf_handle* h, char* buf, size_t n) {
    if (!h || !buf || n == 0) return NF_ERR_PARAM;
    std::snprintf(buf, n, "%s", h->E.err.c_str());
    return NF_OK;
}

nf_status nf_load_density(nf_handle* h, int nx, int ny, int nz, const float* values) {
    if (!h || !values || nx <= 0 || ny <= 0 || nz <= 0) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_load_density");
    h->p.mesh_ext[0] = nx; h->p.mesh_ext[1] = ny; h->p.mesh_ext[2] = nz;
    return h->E.set_density(0, nx, ny, nz, values);
}

nf_status nf_generate(nf_handle* h, nf_gen_stats* stats) {
    if (!h) return NF_ERR_PARAM;
    nf_status s = h->E.generate();
    if (stats) *stats = h->E.gst;
    return s;
}

nf_status nf_autotune(nf_handle* h, nf_tune_result* out) {
    if (!h) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (E.R != 1 && E.adaptive()) return fail(h, NF_ERR_STATE, "adaptive generation runs on single handles");
    int trials = 0;
    // The speed-only settings, applied to every realisation of the handle.
    struct Tune {
        int32_t stencil_radius;
        float round_overshoot, tube_load;
        double two_phase_work;
    };
    auto apply = [&](const Tune& t) {
        for (auto& q : E.prm) {
            q.stencil_radius = t.stencil_radius;
            q.round_overshoot = t.round_overshoot;
            q.tube_load = t.tube_load;
            q.two_phase_work = t.two_phase_work;
        }
        h->p = E.prm[0];
    };
    // Generation time under t: one untimed run (buffers grow to the new
    // sizes), then one timed run (CUDA events inside nf_generate).
    auto time_of = [&](const Tune& t, double* ms) -> nf_status {
        apply(t);
        nf_status s = E.generate();
        if (s == NF_OK) s = E.generate();
        if (s != NF_OK) return s;
        *ms = E.gst.ms;
        ++trials;
        return NF_OK;
    };
    const nf_params& p0 = E.prm[0];
    Tune best{p0.stencil_radius, p0.round_overshoot, p0.tube_load, p0.two_phase_work};
    double t_best = 0;
    nf_status s = time_of(best, &t_best);
    if (s != NF_OK) return s;
    const double ms_first = t_best;
    auto try_value = [&](auto set, auto value) -> nf_status {
        Tune q = best;
        set(q, value);
        double t = 0;
        nf_status st = time_of(q, &t);
        if (st != NF_OK) return st;
        if (t < t_best) { t_best = t; best = q; }
        return NF_OK;
    };
    // the round size: three values besides the one on entry (0: 1.5)
    auto try_overshoot = [&]() -> nf_status {
        const float on_entry = best.round_overshoot > 0 ? best.round_overshoot : 1.5f;
        int n = 0;
        for (float f : {1.25f, 1.5f, 2.0f, 3.0f}) {
            if (f == on_entry || n == 3) continue;
            ++n;
            nf_status st = try_value([](Tune& q, float v) { q.round_overshoot = v; }, f);
            if (st != NF_OK) return st;
        }
        return NF_OK;
    };
    if (E.tube) {  // tube grid: the cell edge (through the load) and the round size
        const float on_entry = best.tube_load > 0 ? best.tube_load : 64.0f;
        for (float l : {32.0f, 48.0f, 64.0f, 96.0f, 128.0f}) {
            if (l == on_entry) continue;
            s = try_value([](Tune& q, float v) { q.tube_load = v; }, l);
            if (s != NF_OK) return s;
        }
        s = try_overshoot();
        if (s != NF_OK) return s;
    } else {
        for (int r : {1, 2}) {
            s = try_value([](Tune& q, int v) { q.stencil_radius = v; }, r);
            if (s != NF_OK) return s;
        }
        s = try_overshoot();
        if (s != NF_OK) return s;
        for (double w : {1e9, 1e10, -1.0}) {
            s = try_value([](Tune& q, double v) { q.two_phase_work = v; }, w);
            if (s != NF_OK) return s;
        }
    }
    // Leave the handle generated under the chosen settings.
    apply(best);
    s = E.generate();
    if (s != NF_OK) return s;
    if (out) {
        out->stencil_radius = best.stencil_radius;
        out->round_overshoot = best.round_overshoot;
        out->two_phase_work = best.two_phase_work;
        out->ms_first = ms_first;
        out->ms_best = t_best;
        out->trials = trials;
        out->tube_load = best.tube_load;
    }
    return NF_OK;
}

nf_status nf_stream_candidates(nf_handle* h, uint64_t k0, uint64_t n, float* x, float* y, float* z, float* cx,
                               float* cy, float* cz, float* l, float* a, float* u, float* rho) {
    if (!h) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_stream_candidates");
    std::vector<float> o(10 * n);
    nf_status s = h->E.stream_dump(k0, n, o.data());
    if (s != NF_OK) return s;
    float* dst[10] = {x, y, z, cx, cy, cz, l, a, u, rho};
    for (int f = 0; f < 10; ++f)
        if (dst[f])
            for (uint64_t i = 0; i < n; ++i) dst[f][i] = o[10 * i + f];
    return NF_OK;
}

nf_status nf_get_rods(nf_handle* h, nf_rods* out) {
    if (!h || !out) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (E.count.empty() || !E.cells_valid) return fail(h, NF_ERR_STATE, "no rods");
    const int rr = h->cur;
    size_t n = E.count[rr];
    const size_t ro = E.hreal[rr].rod_off;
    out->count = n;
    if (out->capacity < n) return NF_ERR_CAPACITY;
    // staged through the handle's pinned host buffer (asynchronous copies at
    // the link's rate), then unpacked into the caller's arrays
    nf_status st = E.ensure_pinned(n * (2 * sizeof(float4) + sizeof(uint64_t)) + 16);
    if (st != NF_OK) return st;
    float4* p = reinterpret_cast<float4*>(E.hpin);
    float4* d = p + n;
    uint64_t* k = reinterpret_cast<uint64_t*>(d + n);
    cudaError_t e = cudaSuccess;
    if (n) {
        e = cudaMemcpyAsync(p, E.pos.p + ro, sizeof(float4) * n, cudaMemcpyDeviceToHost, E.st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d, E.dir.p + ro, sizeof(float4) * n, cudaMemcpyDeviceToHost, E.st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(k, E.sidx.p + ro, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, E.st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(E.st);
    }
    if (e != cudaSuccess) return E.cuda_fail(e, "nf_get_rods");
    const nf::Real& Re = E.hreal[rr];
    // one pass over the staging buffer; no per-element tests when every field is wanted
    if (out->x && out->y && out->z && out->l && out->cx && out->cy && out->cz && out->a && out->stream_index &&
        out->cell) {
        for (size_t i = 0; i < n; ++i) {
            const float4 pi = p[i], di = d[i];
            out->x[i] = pi.x; out->y[i] = pi.y; out->z[i] = pi.z; out->l[i] = pi.w;
            out->cx[i] = di.x; out->cy[i] = di.y; out->cz[i] = di.z; out->a[i] = di.w;
            out->stream_index[i] = k[i];
            out->cell[i] = nf::cell_of(Re, pi.x, pi.y, pi.z);
        }
        return NF_OK;
    }
    for (size_t i = 0; i < n; ++i) {
        if (out->x) out->x[i] = p[i].x;
        if (out->y) out->y[i] = p[i].y;
        if (out->z) out->z[i] = p[i].z;
        if (out->l) out->l[i] = p[i].w;
        if (out->cx) out->cx[i] = d[i].x;
        if (out->cy) out->cy[i] = d[i].y;
        if (out->cz) out->cz[i] = d[i].z;
        if (out->a) out->a[i] = d[i].w;
        if (out->stream_index) out->stream_index[i] = k[i];
        if (out->cell) out->cell[i] = nf::cell_of(Re, p[i].x, p[i].y, p[i].z);
    }
    return NF_OK;
}

nf_status nf_set_rods(nf_handle* h, const nf_rods* in) {
    if (!h || !in || !in->x || !in->y || !in->z || !in->cx || !in->cy || !in->cz || !in->l || !in->a)
        return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_set_rods");
    size_t n = in->count;
    std::vector<float4> p(n), d(n);
    for (size_t i = 0; i < n; ++i) {
        p[i] = make_float4(in->x[i], in->y[i], in->z[i], in->l[i]);
        d[i] = make_float4(in->cx[i], in->cy[i], in->cz[i], in->a[i]);
    }
    return h->E.inject(n, p.data(), d.data(), in->stream_index);
}

nf_status nf_contacts(nf_handle* h, nf_contact_stats* stats) {
    if (!h) return NF_ERR_PARAM;
    nf_status s = h->E.contacts();
    if (stats) *stats = h->E.cst;
    return s;
}

nf_status nf_get_contacts(nf_handle* h, nf_contact_list* out) {
    if (!h || !out) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (!E.contacts_valid) return fail(h, NF_ERR_STATE, "no contacts");
    const int rr = h->cur;
    size_t lo = E.ct_off[rr], n = E.ct_off[rr + 1] - lo;
    out->count = n;
    if (out->capacity < n) return NF_ERR_CAPACITY;
    // staged through the handle's pinned host buffer: doubles, then ids, then images
    nf_status st = E.ensure_pinned(n * (5 * sizeof(double) + 2 * sizeof(uint32_t) + 3) + 16);
    if (st != NF_OK) return st;
    double* t0 = reinterpret_cast<double*>(E.hpin);
    double* t1 = t0 + n;
    double* D = t1 + n;
    double* G = D + n;
    double* S = G + n;
    uint32_t* I = reinterpret_cast<uint32_t*>(S + n);
    uint32_t* J = I + n;
    int8_t* img = reinterpret_cast<int8_t*>(J + n);
    cudaError_t e = cudaSuccess;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, E.st);
    };
    cp(I, E.cI.p + lo, 4 * n); cp(J, E.cJ.p + lo, 4 * n);
    cp(t0, E.ct0.p + lo, 8 * n); cp(t1, E.ct1.p + lo, 8 * n);
    cp(D, E.cD.p + lo, 8 * n); cp(G, E.cG.p + lo, 8 * n); cp(S, E.cS.p + lo, 8 * n);
    cp(img, E.cimg.p + 3 * lo, 3 * n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(E.st);
    if (e != cudaSuccess) return E.cuda_fail(e, "nf_get_contacts");
    const uint32_t off = E.hreal[rr].rod_off;
    if (out->I) for (size_t q = 0; q < n; ++q) out->I[q] = I[q] - off;
    if (out->J) for (size_t q = 0; q < n; ++q) out->J[q] = J[q] >= NF_SNK_ELEC ? J[q] : J[q] - off;
    if (out->tI) for (size_t q = 0; q < n; ++q) out->tI[q] = (float)t0[q];
    if (out->tJ) for (size_t q = 0; q < n; ++q) out->tJ[q] = (float)t1[q];
    if (out->D) std::memcpy(out->D, D, sizeof(double) * n);
    if (out->G) std::memcpy(out->G, G, sizeof(double) * n);
    if (out->S) std::memcpy(out->S, S, sizeof(double) * n);
    if (out->image) std::memcpy(out->image, img, 3 * n);
    return NF_OK;
}

nf_status nf_solve(nf_handle* h, nf_solve_stats* stats) {
    if (!h) return NF_ERR_PARAM;
    nf_status s = h->E.solve();
    if (stats && (int)h->E.solve_st.size() > h->cur) *stats = h->E.solve_st[h->cur];
    return s;
}

nf_status nf_get_voltages(nf_handle* h, double* v, size_t capacity) {
    if (!h || !v) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_get_voltages");
    nf::Engine& E = h->E;
    if (!E.solve_valid) return fail(h, NF_ERR_STATE, "no solution");
    size_t n = E.int_valid ? E.int_count[0] : E.count[0];
    if (capacity < n) return NF_ERR_CAPACITY;
    cudaError_t e = cudaMemcpyAsync(v, E.volt.p, sizeof(double) * n, cudaMemcpyDeviceToHost, E.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(E.st);
    if (e != cudaSuccess) return E.cuda_fail(e, "nf_get_voltages");
    return NF_OK;
}

nf_status nf_adjoint(nf_handle* h, float* dG_dend, size_t capacity, double* dG_dlambda, double* dG_dG0) {
    if (!h) return NF_ERR_PARAM;
    if (h->E.int_valid)
        return fail(h, NF_ERR_UNSUPPORTED, "the adjoint covers the contact network (run nf_contacts again)");
    if (h->E.prm[0].elec_buffer && h->E.prm[0].field_dir)
        return fail(h, NF_ERR_UNSUPPORTED, "the adjoint covers plane electrodes (ELEC_BUFFER 0)");
    return h->E.adjoint(h->cur, dG_dend, capacity, dG_dlambda, dG_dG0);
}

nf_status nf_internal_network(nf_handle* h, nf_internal_stats* stats) {
    if (!h) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (E.R != 1) return fail(h, NF_ERR_STATE, "the internal network is built on a single-realisation handle");
    nf_status s = E.internal_network();
    if (s != NF_OK) return s;
    if (stats) {
        stats->contact_ends = E.int_full;
        stats->nodes = E.int_nodes;
        stats->segments = E.int_segs;
    }
    return NF_OK;
}

nf_status nf_get_internal_network(nf_handle* h, nf_internal_net* out) {
    if (!h || !out) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_get_internal_network");
    nf::Engine& E = h->E;
    if (!E.int_valid) return fail(h, NF_ERR_STATE, "no internal network: run nf_internal_network first");
    const size_t nn = E.int_nodes, ns = E.int_segs, ne = E.ct_off[1];
    out->n_nodes = nn;
    out->n_segments = ns;
    out->n_edges = ne;
    const size_t need = std::max(nn, std::max(ns, ne));
    const bool any = out->node_rod || out->node_t || out->seg_i || out->seg_j || out->seg_l || out->seg_g ||
                     out->edge_i || out->edge_j;
    if (!any) return NF_OK;
    if (out->capacity < need) return NF_ERR_CAPACITY;
    struct Copy { void* dst; const void* src; size_t bytes; };
    const Copy cp[] = {{out->node_rod, E.inrod.p, 4 * nn}, {out->node_t, E.int_t.p, 8 * nn},
                       {out->seg_i, E.ieI.p + ne, 4 * ns}, {out->seg_j, E.ieJ.p + ne, 4 * ns},
                       {out->seg_l, E.iseg_l.p, 8 * ns}, {out->seg_g, E.ieG.p + ne, 8 * ns},
                       {out->edge_i, E.ieI.p, 4 * ne}, {out->edge_j, E.ieJ.p, 4 * ne}};
    cudaError_t e = cudaSuccess;
    for (const Copy& c : cp)
        if (c.dst && c.bytes && e == cudaSuccess) e = cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, E.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(E.st);
    if (e != cudaSuccess) return E.cuda_fail(e, "nf_get_internal_network");
    return NF_OK;
}

nf_status nf_write_internal_coo(nf_handle* h, const char* dir) {
    if (!h || !dir) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_write_internal_coo");
    nf::Engine& E = h->E;
    if (!E.int_valid) return fail(h, NF_ERR_STATE, "no internal network: run nf_internal_network first");
    nf_internal_net net{};
    nf_status s = nf_get_internal_network(h, &net);
    if (s != NF_OK) return s;
    const size_t nn = net.n_nodes, ns = net.n_segments, ne = net.n_edges;
    std::vector<uint32_t> nrod(nn), si(ns), sj(ns), ei(ne), ej(ne);
    std::vector<double> nt(nn), sl(ns), sg(ns);
    net.capacity = std::max(nn, std::max(ns, ne));
    net.node_rod = nrod.data(); net.node_t = nt.data();
    net.seg_i = si.data(); net.seg_j = sj.data(); net.seg_l = sl.data(); net.seg_g = sg.data();
    net.edge_i = ei.data(); net.edge_j = ej.data();
    if (net.capacity && (s = nf_get_internal_network(h, &net)) != NF_OK) return s;
    std::vector<uint32_t> I(ne), J(ne);
    std::vector<double> D(ne), S(ne);
    nf_contact_list c{};
    c.capacity = ne;
    c.I = I.data(); c.J = J.data(); c.D = D.data(); c.S = S.data();
    if ((s = nf_get_contacts(h, &c)) != NF_OK) return s;
    std::vector<float> rad(E.count[0]);
    nf_rods r{};
    r.capacity = rad.size();
    r.a = rad.data();
    if ((s = nf_get_rods(h, &r)) != NF_OK) return s;
    auto open = [&](const char* name, const char* header, std::ofstream& o) {
        o.open(std::string(dir) + "/" + name);
        if (o.is_open()) o << header;
        return o.is_open();
    };
    std::ofstream o;
    // Nodes.tbl.dat: node, rod, t (save_coo with one data column)
    if (!open("Nodes.tbl.dat", "#\tI\tJ\tData\n", o)) return NF_ERR_IO;
    for (size_t k = 0; k < nn; ++k) o << "\t" << k << "\t" << nrod[k] << "\t" << (float)nt[k] << "\n";
    if (!o.good()) return NF_ERR_IO;
    o.close();
    // segment.LA.coo: i, j, L, a
    if (!open("segment.LA.coo", "#\tI\tJ\tData1\tData2\n", o)) return NF_ERR_IO;
    for (size_t k = 0; k < ns; ++k)
        o << "\t" << si[k] << "\t" << sj[k] << "\t" << (float)sl[k] << "\t" << rad[nrod[si[k]]] << "\n";
    if (!o.good()) return NF_ERR_IO;
    o.close();
    // internal / sink / source .DS.coo: node pairs with D and S, each block sorted
    // by its node pair (electrode contacts written as (electrode id, node)).
    const size_t nint = E.ct_int[0], nsnk = E.ct_snk[0];
    const size_t b[4] = {0, nint, nint + nsnk, ne};
    const char* names[3] = {"internal.DS.coo", "sink.DS.coo", "source.DS.coo"};
    for (int f = 0; f < 3; ++f) {
        std::vector<size_t> ord;
        for (size_t q = b[f]; q < b[f + 1]; ++q) ord.push_back(q);
        auto key = [&](size_t q) {
            return f == 0 ? std::make_pair(ei[q], ej[q]) : std::make_pair(ej[q], ei[q]);
        };
        std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return key(x) < key(y); });
        if (!open(names[f], "#\tI\tJ\tData1\tData2\n", o)) return NF_ERR_IO;
        for (size_t q : ord) {
            const std::pair<uint32_t, uint32_t> k = key(q);
            o << "\t" << k.first << "\t" << k.second << "\t" << (float)D[q] << "\t" << (float)S[q] << "\n";
        }
        if (!o.good()) return NF_ERR_IO;
        o.close();
    }
    return NF_OK;
}

nf_status nf_set_orientation(nf_handle* h, int32_t mode, float kappa, float pref_phi, float pref_theta) {
    if (!h) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    std::vector<nf_params> ps = E.prm;
    for (nf_params& p : ps) {
        p.orient_mode = mode;
        p.vmf_kappa = kappa;
        p.pref_ort[0] = pref_phi;
        p.pref_ort[1] = pref_theta;
        std::string why;
        if (mode != NF_ORIENT_ISOTROPIC && mode != NF_ORIENT_VMF) return fail(h, NF_ERR_PARAM, "unknown orientation mode");
        if (!std::isfinite(pref_phi) || !std::isfinite(pref_theta)) return fail(h, NF_ERR_PARAM, "axis angles must be finite");
        nf_status s = validate(p, &why);
        if (s != NF_OK) return fail(h, s, why);
    }
    E.prm = ps;
    return E.setup();  // the device descriptors follow at once
}

nf_status nf_orientation_laws(nf_handle* h, size_t cap, int32_t ext[3], float* axis, float* kappa, size_t* cells) {
    if (!h) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_orientation_laws");
    nf_status s = h->E.orientation_laws(cap, ext, axis, kappa, cells);
    if (s != NF_OK) return fail(h, s, h->E.err);
    return NF_OK;
}

nf_status nf_reduce(nf_handle* h, int32_t min_contacts, nf_reduce_stats* stats) {
    if (!h) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_reduce");
    if (min_contacts < 0) return fail(h, NF_ERR_PARAM, "min_contacts must be >= 0");
    nf_reduce_stats st{};
    nf_status s = h->E.prune(min_contacts, &st);
    if (stats) *stats = st;
    return s;
}

nf_status nf_stat_nematic(nf_handle* h, const double axis[3], double* S) {
    if (!h || !axis || !S) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_stat_nematic");
    return h->E.stat_nematic(axis, S);
}

nf_status nf_stat_phitheta(nf_handle* h, int32_t bins_phi, int32_t bins_theta, uint64_t* hist) {
    if (!h || !hist) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_stat_phitheta");
    return h->E.stat_phitheta(bins_phi, bins_theta, hist);
}

nf_status nf_stat_pairs(nf_handle* h, int32_t bins, uint64_t* hist, uint32_t* per_rod, size_t capacity,
                        nf_pair_stats* stats) {
    if (!h) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_stat_pairs");
    return h->E.stat_pairs(bins, hist, per_rod, capacity, stats);
}

namespace {
// Rods of realisation 0 on the host.
nf_status host_rods(nf_handle* h, std::vector<float>* f) {
    nf_rods r{};
    nf_status s = nf_get_rods(h, &r);
    if (s != NF_OK && s != NF_ERR_CAPACITY) return s;
    const size_t n = r.count;
    for (int k = 0; k < 8; ++k) f[k].assign(n, 0.f);
    r.capacity = n;
    r.x = f[0].data(); r.y = f[1].data(); r.z = f[2].data();
    r.cx = f[3].data(); r.cy = f[4].data(); r.cz = f[5].data();
    r.l = f[6].data(); r.a = f[7].data();
    return nf_get_rods(h, &r);
}
}  // namespace

nf_status nf_write_ort_vtk(nf_handle* h, const char* path) {
    if (!h || !path) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_write_ort_vtk");
    std::vector<float> f[8];
    nf_status s = host_rods(h, f);
    if (s != NF_OK) return s;
    s = nf_format_write_ort_vtk(path, f[0].size(), f[3].data(), f[4].data(), f[5].data());
    return s == NF_OK ? s : fail(h, s, path);
}

nf_status nf_write_lmp(nf_handle* h, const char* path, double density) {
    if (!h || !path) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_write_lmp");
    std::vector<float> f[8];
    nf_status s = host_rods(h, f);
    if (s != NF_OK) return s;
    s = nf_format_write_lmp(path, f[0].size(), f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(),
                            f[5].data(), f[6].data(), f[7].data(), h->E.prm[0].box, density);
    return s == NF_OK ? s : fail(h, s, path);
}

nf_status nf_format_write_rho(const char* path, int32_t bx, int32_t by, const uint64_t* hist) {
    if (!path || !hist || bx <= 0 || by <= 0) return NF_ERR_PARAM;
    std::ofstream o(path, std::ios::out | std::ios::trunc);
    if (!o) return NF_ERR_IO;
    o << "rho = {";
    for (int j = 0; j < by; ++j) {
        o << "\t{";
        for (int i = 0; i < bx; ++i) {
            o << std::setw(12) << hist[i + (size_t)j * bx];
            if (i != bx - 1) o << ",";
        }
        o << "}";
        if (j != by - 1) o << "," << std::endl << "\t";
    }
    o << "}";
    return o.good() ? NF_OK : NF_ERR_IO;
}

nf_status nf_format_write_gamma(const char* path, int32_t bins, const uint64_t* hist) {
    if (!path || !hist || bins <= 0) return NF_ERR_PARAM;
    std::ofstream o(path, std::ios::out | std::ios::trunc);
    if (!o) return NF_ERR_IO;
    o << "gamma={\t";
    for (int i = 0; i < bins - 1; ++i) o << std::setw(10) << std::setprecision(7) << (double)hist[i] << "," << std::endl;
    o << std::setw(10) << std::setprecision(7) << (double)hist[bins - 1] << "\t}" << std::endl;
    return o.good() ? NF_OK : NF_ERR_IO;
}

void nf_ac_params_default(nf_ac_params* p) {
    if (!p) return;
    *p = nf_ac_params{};
    // the constants of tools/kirchhoff/kirchhoff.py:55-68 (lengths in um)
    p->r_cnt = 4.75e-3;
    p->l_cnt = 1.5;
    p->phi_ev = 3.5;
    p->eps_r = 2.9;
    p->delta_min = 0.34e-3;
    p->delta_tun = 1.1e-3;
    p->delta_eff = 50e-3;
    p->c_min = 0.005;
    p->l_box = 1.0;
    p->own_radii = 0;
    p->tol = 1e-10;
}

size_t nf_ac_frequencies(double log_df, int n_patch, int patch_id, double* freq, size_t capacity) {
    if (!(log_df > 0) || n_patch < 1 || patch_id < 0 || patch_id >= n_patch) return 0;
    // kirchhoff.py:72-79,176: N = int(16 / log_df) + 1 points from 10^-2 Hz,
    // patch = ceil(N / n_patch) points from logF_min = -2 + patch_id patch log_df
    const long nf = (long)((14.0 - (-2.0)) / log_df) + 1;
    const long patch = (long)std::ceil(nf * 1.0 / n_patch);
    const double lo = -2.0 + patch_id * patch * log_df;
    for (long x = 0; x < patch && (size_t)x < capacity; ++x)
        if (freq) freq[x] = std::pow(10.0, log_df * x + lo);
    return (size_t)patch;
}

nf_status nf_ac_spectrum(nf_handle* h, const nf_ac_net* net, const nf_ac_params* p, const double* freq,
                         size_t n_freq, nf_ac_point* out, nf_ac_stats* stats) {
    if (!h || !p || (n_freq && (!freq || !out))) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (!(p->r_cnt > 0) || !(p->l_cnt > 0) || !(p->phi_ev > 0) || !(p->eps_r > 0) || !(p->delta_min > 0) ||
        !(p->delta_tun >= 0) || !(p->delta_eff > 0) || !(p->c_min >= 0) || !(p->l_box > 0) ||
        (p->own_radii != 0 && p->own_radii != 1) || p->method < 0 || p->method > 2)
        return fail(h, NF_ERR_PARAM, "AC parameters out of range");
    for (size_t f = 0; f < n_freq; ++f)
        if (!(freq[f] > 0) || !std::isfinite(freq[f])) return fail(h, NF_ERR_PARAM, "frequencies must be positive");
    if (!net) {
        if (E.R != 1) return fail(h, NF_ERR_STATE, "the AC spectrum runs on a single-realisation handle");
        if (!E.contacts_valid) return fail(h, NF_ERR_STATE, "no contacts: run nf_contacts first");
    } else {
        if (p->own_radii) return fail(h, NF_ERR_PARAM, "own_radii needs the handle's own network");
        const uint64_t n = net->n_nodes;
        if (n == 0 || n >= NF_SNK_ELEC) return fail(h, NF_ERR_PARAM, "n_nodes out of range");
        if ((net->n_segments && (!net->seg_i || !net->seg_j || !net->seg_l || !net->seg_a)) ||
            (net->n_contacts && (!net->ct_i || !net->ct_j || !net->ct_d || !net->ct_s)))
            return fail(h, NF_ERR_PARAM, "null network array");
        if (net->n_segments + net->n_contacts >= (1ull << 31)) return fail(h, NF_ERR_PARAM, "network too large");
        for (uint64_t s = 0; s < net->n_segments; ++s)
            if (net->seg_i[s] >= n || net->seg_j[s] >= n || net->seg_i[s] == net->seg_j[s] ||
                !(net->seg_l[s] > 0) || !(net->seg_a[s] > 0))
                return fail(h, NF_ERR_PARAM, "segment out of range");
        for (uint64_t c = 0; c < net->n_contacts; ++c) {
            const uint32_t j = net->ct_j[c];
            if (net->ct_i[c] >= n || (j >= n && j < NF_SNK_ELEC) || j == net->ct_i[c] || !std::isfinite(net->ct_d[c]) ||
                !std::isfinite(net->ct_s[c]))
                return fail(h, NF_ERR_PARAM, "contact out of range");
        }
    }
    if (n_freq == 0) return NF_OK;
    return E.ac_spectrum(net, *p, freq, n_freq, out, stats);
}

// Parameters of a batch: per-realisation density files read, every
// realisation validated, one electrode model when buffer layers are used.
static nf_status prepare_batch(const nf_params* params, int n, std::vector<nf_params>* ps,
                               std::vector<std::vector<float>>* meshes, std::vector<const float*>* mp,
                               std::string* why) {
    ps->assign(params, params + n);
    for (int r = 0; r < n; ++r)  // the adaptive generation runs on single-realisation handles
        if ((*ps)[r].self_align_step > 0 || (*ps)[r].clust_flag) {
            *why = "adaptive generation runs on single-realisation handles";
            return NF_ERR_UNSUPPORTED;
        }
    for (int r = 1; r < n; ++r)  // one electrode model and field axis per engine when buffer layers are used
        if (((*ps)[r].elec_buffer || (*ps)[0].elec_buffer) &&
            ((*ps)[r].elec_buffer != (*ps)[0].elec_buffer || (*ps)[r].field_dir != (*ps)[0].field_dir)) {
            *why = "a batch with buffer-layer electrodes needs one electrode model and field axis";
            return NF_ERR_PARAM;
        }
    meshes->assign(n, {});
    mp->assign(n, nullptr);
    for (int r = 0; r < n; ++r) {
        nf_params& q = (*ps)[r];
        if (q.density_file[0]) {
            int ext[3];
            float dim[3];
            if (!read_density(q.density_file, ext, dim, &(*meshes)[r])) {
                *why = std::string("cannot read density file ") + q.density_file;
                return NF_ERR_FORMAT;
            }
            for (int d = 0; d < 3; ++d) { q.box[d] = dim[d]; q.mesh_ext[d] = ext[d]; }
            (*mp)[r] = (*meshes)[r].data();
        } else {
            q.mesh_ext[0] = q.mesh_ext[1] = q.mesh_ext[2] = 0;
        }
        nf_status s = validate(q, why);
        if (s != NF_OK) return s;
    }
    return NF_OK;
}

nf_status nf_create_batch(const nf_params* params, int n, nf_handle** out) {
    if (!params || n <= 0 || !out) return NF_ERR_PARAM;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NF_ERR_NO_DEVICE;
    std::vector<nf_params> ps;
    std::vector<std::vector<float>> meshes;
    std::vector<const float*> mp;
    std::string why;
    nf_status s = prepare_batch(params, n, &ps, &meshes, &mp, &why);
    if (s != NF_OK) return s;
    nf_handle* h = new (std::nothrow) nf_handle();
    if (!h) return NF_ERR_ALLOC;
    h->p = ps[0];
    s = h->E.init(ps.data(), n, mp);
    if (s != NF_OK) { delete h; return s; }
    *out = h;
    return NF_OK;
}

nf_status nf_select(nf_handle* h, int32_t r) {
    if (!h) return NF_ERR_PARAM;
    if (r < 0 || r >= h->E.R) return fail(h, NF_ERR_PARAM, "realisation index out of range");
    h->cur = r;
    return NF_OK;
}

nf_status nf_batch_results(nf_handle* h, nf_batch_result* out, int32_t n) {
    if (!h || !out || n != h->E.R) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (!E.solve_valid || (int)E.solve_st.size() != n) return fail(h, NF_ERR_STATE, "no solution");
    for (int r = 0; r < n; ++r) {
        const nf_solve_stats& S = E.solve_st[r];
        out[r].accepted = E.count[r];
        out[r].contacts = E.ct_int[r];
        out[r].G_eff = S.G_eff;
        out[r].residual = S.residual;
        out[r].percolating = S.percolating;
        out[r].status = (S.n_active > 0 && !(S.residual <= E.prm[r].solve_tol)) ? NF_ERR_NOT_CONVERGED : NF_OK;
    }
    return NF_OK;
}

nf_status nf_batch_run(const nf_params* params, int n, nf_batch_result* out, nf_batch_stats* stats) {
    if (!params || n <= 0 || !out) return NF_ERR_PARAM;
    nf_handle* h = nullptr;
    nf_status s = nf_create_batch(params, n, &h);
    if (s != NF_OK) return s;
    nf::Engine& E = h->E;
    nf::EventPair ev;
    if (ev.create() != cudaSuccess) { nf_destroy(h); return NF_ERR_CUDA; }
    cudaEventRecord(ev.a, E.st);
    // with AUTOTUNE the tuner's last generation (under the settings it keeps)
    // is the batch's generation
    s = params[0].autotune == 1 ? nf_autotune(h, nullptr) : E.generate();
    if (s == NF_OK) s = E.contacts();
    nf_status ss = NF_OK;
    if (s == NF_OK) ss = E.solve();
    if (s == NF_OK && (ss == NF_OK || ss == NF_ERR_NOT_CONVERGED)) {
        s = nf_batch_results(h, out, n);
        if (s == NF_OK && stats) {
            float ms = 0;
            cudaEventRecord(ev.b, E.st);
            cudaEventSynchronize(ev.b);
            cudaEventElapsedTime(&ms, ev.a, ev.b);
            stats->n = n;
            stats->rounds = E.gst.rounds;
            stats->rods = E.gst.accepted;
            stats->contacts = E.cst.contacts;
            stats->ms = ms;
        }
    } else if (s == NF_OK) {
        s = ss;
    }
    nf_destroy(h);
    return s;
}

uint64_t nf_kernel_launches(void) { return nf::g_launches; }
uint64_t nf_allocations(void) { return nf::g_allocs; }

nf_status nf_set_kernel_timing(nf_handle* h, int on) {
    if (!h) return NF_ERR_PARAM;
    nf_status s = h->E.tresolve();
    if (s != NF_OK) return s;
    for (auto& k : h->E.kt) { k.ms = 0; k.n = 0; k.bytes = 0; k.flops = 0; }
    h->E.timing = on != 0;
    // Create the events up front so recording them costs no host-side creation.
    while (on && h->E.evpool.size() < 8192) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) break;
        h->E.evpool.push_back(e);
    }
    return NF_OK;
}

nf_status nf_kernel_time(nf_handle* h, const char* kernel, double* ms, uint64_t* launches, double* bytes,
                         double* flops) {
    if (!h || !kernel) return NF_ERR_PARAM;
    static const char* names[nf::KT_N] = {"stream", "old_test", "conflicts", "resolve", "ct_pairs", "screen", "cg"};
    int k = -1;
    for (int i = 0; i < nf::KT_N; ++i)
        if (!std::strcmp(kernel, names[i])) k = i;
    if (k < 0) return NF_ERR_PARAM;
    nf_status s = h->E.tresolve();
    if (s != NF_OK) return s;
    if (ms) *ms = h->E.kt[k].ms;
    if (launches) *launches = h->E.kt[k].n;
    if (bytes) *bytes = h->E.kt[k].bytes;
    if (flops) *flops = h->E.kt[k].flops;
    return NF_OK;
}

// ---------------------------------------------------------------------------
// Files.
// ---------------------------------------------------------------------------
nf_status nf_format_write_ort_vtk(const char* path, size_t n, const float* cx, const float* cy, const float* cz) {
    if (!path || (n && (!cx || !cy || !cz))) return NF_ERR_PARAM;
    // write_CNT_ORTvtk (src/IO.cpp:77-99): the directions as points
    std::ofstream o(path, std::ios::out | std::ios::trunc);
    if (!o) return NF_ERR_IO;
    o << "# vtk DataFile Version 2.0" << std::endl << "CUDA generated CNTs" << std::endl << "ASCII" << std::endl
      << "DATASET UNSTRUCTURED_GRID" << std::endl << "POINTS " << n << " float" << std::endl;
    for (size_t i = 0; i < n; ++i)
        o << std::setw(15) << std::setprecision(6) << cx[i] << std::setw(15) << std::setprecision(6) << cy[i]
          << std::setw(15) << std::setprecision(6) << cz[i] << std::endl;
    return o.good() ? NF_OK : NF_ERR_IO;
}

nf_status nf_format_write_lmp(const char* path, size_t n, const float* x, const float* y, const float* z,
                              const float* cx, const float* cy, const float* cz, const float* l, const float* a,
                              const float box[3], double density) {
    if (!path || !box || (n && (!x || !y || !z || !cx || !cy || !cz || !l || !a))) return NF_ERR_PARAM;
    // write_CNTlmp (src/IO.cpp:100-146): LAMMPS data file of ellipsoids
    std::ofstream o(path, std::ios::out | std::ios::trunc);
    if (!o) return NF_ERR_IO;
    o << "CUDA generated aspherical particles" << std::endl << std::endl << n << " atoms" << std::endl
      << 1 << " atom types" << std::endl << n << " ellipsoids" << std::endl << std::endl
      << 0.0f << ' ' << box[0] << " xlo xhi" << std::endl << 0.0f << ' ' << box[1] << " ylo yhi" << std::endl
      << 0.0f << ' ' << box[2] << " zlo zhi" << std::endl << std::endl << "Atoms" << std::endl << std::endl;
    for (size_t i = 0; i < n; ++i)
        o << i + 1 << ' ' << 1 << ' ' << 1 << ' ' << (float)density << std::setw(12) << std::setprecision(6)
          << x[i] << std::setw(12) << std::setprecision(6) << y[i] << std::setw(12) << std::setprecision(6)
          << z[i] << std::endl;
    o << std::endl << "Ellipsoids" << std::endl << std::endl;
    // quaternion of the rotation from x to c: axis (0, -cz, cy), angle acos(cx)
    for (size_t i = 0; i < n; ++i) {
        const float sh = sqrtf((1 - cx[i]) / 2);
        o << i + 1 << std::setw(12) << std::setprecision(6) << l[i] + 2 * a[i] << std::setw(12)
          << std::setprecision(6) << 2 * a[i] << std::setw(12) << std::setprecision(6) << 2 * a[i] << std::setw(15)
          << std::setprecision(6) << sqrtf((1 + cx[i]) / 2) << std::setw(15) << std::setprecision(6) << 0.0f
          << std::setw(15) << std::setprecision(6) << -cz[i] * sh << std::setw(15) << std::setprecision(6)
          << +cy[i] * sh << std::endl;
    }
    return o.good() ? NF_OK : NF_ERR_IO;
}

nf_status nf_format_write_vtk(const char* path, size_t n, const float* x, const float* y, const float* z,
                              const float* cx, const float* cy, const float* cz, const float* l, const float* a,
                              const float* k) {
    if (!path || (n && (!x || !y || !z || !cx || !cy || !cz || !l || !a || !k))) return NF_ERR_PARAM;
    // write_CNTvtk (src/IO.cpp:38-76)
    std::ofstream v(path, std::ios::out | std::ios::trunc);
    if (!v.is_open()) return NF_ERR_IO;
    v << "# vtk DataFile Version 2.0" << std::endl;
    v << "CUDA generated CNTs" << std::endl;
    v << "ASCII" << std::endl;
    v << "DATASET UNSTRUCTURED_GRID" << std::endl;
    v << "POINTS " << n << " float" << std::endl;
    for (size_t i = 0; i < n; ++i)
        v << std::setw(12) << std::setprecision(6) << x[i] << std::setw(12) << std::setprecision(6) << y[i]
          << std::setw(12) << std::setprecision(6) << z[i] << std::endl;
    v << "POINT_DATA " << n << std::endl;
    v << "VECTORS CNT float" << std::endl;
    for (size_t i = 0; i < n; ++i)
        v << std::setw(15) << std::setprecision(6) << cx[i] << std::setw(15) << std::setprecision(6) << cy[i]
          << std::setw(15) << std::setprecision(6) << cz[i] << std::endl;
    v << "SCALARS LAK float 3" << std::endl;
    v << "LOOKUP_TABLE default" << std::endl;
    for (size_t i = 0; i < n; ++i)
        v << std::setw(12) << std::setprecision(6) << l[i] << std::setw(12) << std::setprecision(6) << a[i]
          << std::setw(12) << std::setprecision(6) << k[i] << std::endl;
    return v.good() ? NF_OK : NF_ERR_IO;
}

nf_status nf_format_write_state_bin(const char* path, const nf_state_header* hd, const int16_t* occ,
                                    const int32_t* addr, const float* planes) {
    if (!path || !hd) return NF_ERR_PARAM;
    size_t cells = (size_t)hd->ext[0] * hd->ext[1] * hd->ext[2];
    if ((cells && (!occ || !addr)) || (hd->ttl > 0 && !planes)) return NF_ERR_PARAM;
    // save_state_BIN (src/stateSR.cpp:54-89)
    std::ofstream o(path, std::ios::out | std::ios::binary);
    if (!o.is_open()) return NF_ERR_IO;
    o.write((const char*)hd->phys_dim, 3 * sizeof(float));
    o.write((const char*)hd->edge, 3 * sizeof(float));
    o.write((const char*)hd->ext, 3 * sizeof(int32_t));
    o.write((const char*)&hd->l, sizeof(float));
    o.write((const char*)&hd->a, sizeof(float));
    o.write((const char*)&hd->ttl, sizeof(int32_t));
    o.write((const char*)&hd->num, sizeof(int32_t));
    o.write((const char*)&hd->tol, sizeof(float));
    o.write((const char*)occ, cells * sizeof(int16_t));
    o.write((const char*)addr, cells * sizeof(int32_t));
    o.write((const char*)planes, 9ull * hd->ttl * sizeof(float));
    return o.good() ? NF_OK : NF_ERR_IO;
}

nf_status nf_format_read_state_bin(const char* path, nf_state_header* hd, int16_t* occ, int32_t* addr,
                                   float* planes, size_t cells_cap, size_t planes_cap) {
    if (!path || !hd) return NF_ERR_PARAM;
    // read_state_BIN (src/stateSR.cpp:90-134)
    std::ifstream f(path, std::ios::in | std::ios::binary);
    if (!f.is_open()) return NF_ERR_IO;
    f.read((char*)hd->phys_dim, 3 * sizeof(float));
    f.read((char*)hd->edge, 3 * sizeof(float));
    f.read((char*)hd->ext, 3 * sizeof(int32_t));
    f.read((char*)&hd->l, sizeof(float));
    f.read((char*)&hd->a, sizeof(float));
    f.read((char*)&hd->ttl, sizeof(int32_t));
    f.read((char*)&hd->num, sizeof(int32_t));
    f.read((char*)&hd->tol, sizeof(float));
    if (!f.good()) return NF_ERR_FORMAT;
    if (hd->ext[0] <= 0 || hd->ext[1] <= 0 || hd->ext[2] <= 0 || hd->ttl < 0 || hd->num < 0) return NF_ERR_FORMAT;
    size_t cells = (size_t)hd->ext[0] * hd->ext[1] * hd->ext[2];
    if (!occ && !addr && !planes) return NF_OK;
    if (cells_cap < cells || planes_cap < 9ull * hd->ttl) return NF_ERR_CAPACITY;
    std::vector<int16_t> o(cells);
    std::vector<int32_t> a(cells);
    f.read((char*)o.data(), cells * sizeof(int16_t));
    f.read((char*)a.data(), cells * sizeof(int32_t));
    std::vector<float> pl(9ull * hd->ttl);
    f.read((char*)pl.data(), pl.size() * sizeof(float));
    if (!f.good()) return NF_ERR_FORMAT;
    if (occ) std::copy(o.begin(), o.end(), occ);
    if (addr) std::copy(a.begin(), a.end(), addr);
    if (planes) std::copy(pl.begin(), pl.end(), planes);
    return NF_OK;
}

// Rods of the handle grouped by cell (the repacked layout of simPrms::repack,
// src/simPrms.cpp:691-743), k = global cell id (set_k2dmnIdx, src/simPrms_device.cu:7-39).
static nf_status cell_layout(nf_handle* h, nf_state_header* hd, std::vector<int16_t>* occ, std::vector<int32_t>* addr,
                             std::vector<float>* planes, std::vector<uint32_t>* order) {
    nf::Engine& E = h->E;
    size_t n = E.count.empty() ? 0 : E.count[0];
    std::vector<float> x(n), y(n), z(n), cx(n), cy(n), cz(n), l(n), a(n);
    std::vector<uint32_t> cell(n);
    nf_rods r{};
    r.capacity = n;
    r.x = x.data(); r.y = y.data(); r.z = z.data(); r.cx = cx.data(); r.cy = cy.data(); r.cz = cz.data();
    r.l = l.data(); r.a = a.data(); r.cell = cell.data();
    nf_status s = nf_get_rods(h, &r);
    if (s != NF_OK) return s;
    const nf::Real& Re = E.hreal[0];
    size_t ncell = (size_t)Re.n[0] * Re.n[1] * Re.n[2];
    occ->assign(ncell, 0);
    addr->assign(ncell, 0);
    std::vector<uint32_t> cnt(ncell, 0);
    for (size_t i = 0; i < n; ++i) ++cnt[cell[i]];
    for (size_t c = 0; c < ncell; ++c) {
        if (cnt[c] > 32767) return fail(h, NF_ERR_OVERFLOW, "cell occupancy exceeds the short range of output.bin");
        (*occ)[c] = (int16_t)cnt[c];
        (*addr)[c] = (int32_t)(cnt[c] + (c ? (*addr)[c - 1] : 0));
    }
    order->resize(n);
    std::vector<uint32_t> cur(ncell, 0);
    for (size_t i = 0; i < n; ++i) {
        uint32_t c = cell[i];
        uint32_t q = (c ? (*addr)[c - 1] : 0) + cur[c]++;
        (*order)[q] = (uint32_t)i;
    }
    planes->assign(9 * n, 0.0f);
    for (size_t q = 0; q < n; ++q) {
        uint32_t i = (*order)[q];
        float v[9] = {x[i], y[i], z[i], cx[i], cy[i], cz[i], l[i], a[i], (float)cell[i]};
        for (int f = 0; f < 9; ++f) (*planes)[f * n + q] = v[f];
    }
    for (int d = 0; d < 3; ++d) {
        hd->phys_dim[d] = Re.L[d];
        hd->ext[d] = Re.n[d];
        hd->edge[d] = Re.L[d] / Re.n[d];
    }
    hd->l = h->p.l;
    hd->a = h->p.a;
    hd->ttl = (int32_t)n;
    hd->num = (int32_t)n;
    hd->tol = h->p.tol;
    return NF_OK;
}

nf_status nf_write_vtk(nf_handle* h, const char* path) {
    if (!h || !path) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_write_vtk");
    nf_state_header hd;
    std::vector<int16_t> occ;
    std::vector<int32_t> addr;
    std::vector<float> pl;
    std::vector<uint32_t> order;
    nf_status s = cell_layout(h, &hd, &occ, &addr, &pl, &order);
    if (s != NF_OK) return s;
    size_t n = hd.num;
    const float* P = pl.data();
    return nf_format_write_vtk(path, n, P, P + n, P + 2 * n, P + 3 * n, P + 4 * n, P + 5 * n, P + 6 * n, P + 7 * n,
                               P + 8 * n);
}

nf_status nf_write_state_bin(nf_handle* h, const char* path) {
    if (!h || !path) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_write_state_bin");
    nf_state_header hd;
    std::vector<int16_t> occ;
    std::vector<int32_t> addr;
    std::vector<float> pl;
    std::vector<uint32_t> order;
    nf_status s = cell_layout(h, &hd, &occ, &addr, &pl, &order);
    if (s != NF_OK) return s;
    return nf_format_write_state_bin(path, &hd, occ.data(), addr.data(), pl.data());
}

nf_status nf_read_state_bin(nf_handle* h, const char* path) {
    if (!h || !path) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_read_state_bin");
    nf_state_header hd;
    nf_status s = nf_format_read_state_bin(path, &hd, nullptr, nullptr, nullptr, 0, 0);
    if (s != NF_OK) return s;
    size_t cells = (size_t)hd.ext[0] * hd.ext[1] * hd.ext[2];
    std::vector<int16_t> occ(cells);
    std::vector<int32_t> addr(cells);
    std::vector<float> pl(9ull * hd.ttl);
    s = nf_format_read_state_bin(path, &hd, occ.data(), addr.data(), pl.data(), cells, pl.size());
    if (s != NF_OK) return s;
    // Valid slots of cell c: [Addr[c-1], Addr[c-1] + Occ[c]).
    std::vector<float4> p, d;
    size_t ttl = hd.ttl;
    for (size_t c = 0; c < cells; ++c) {
        size_t b = c ? (size_t)addr[c - 1] : 0;
        for (int k = 0; k < occ[c]; ++k) {
            size_t q = b + k;
            if (q >= ttl) return NF_ERR_FORMAT;
            p.push_back(make_float4(pl[q], pl[ttl + q], pl[2 * ttl + q], pl[6 * ttl + q]));
            d.push_back(make_float4(pl[3 * ttl + q], pl[4 * ttl + q], pl[5 * ttl + q], pl[7 * ttl + q]));
        }
    }
    // the box, rod length, radius and TOL travel with the state, as
    // read_state_BIN (src/stateSR.cpp:96-103) restores physDim, l, a and TOL
    if (!(hd.l > 0) || !(hd.a > 0) || !(hd.tol > 0) || !std::isfinite(hd.l) || !std::isfinite(hd.a) ||
        !std::isfinite(hd.tol))
        return fail(h, NF_ERR_FORMAT, "output.bin header: l, a and TOL must be positive");
    for (nf_params* q : {&h->p, &h->E.prm[0]}) {
        for (int k = 0; k < 3; ++k) q->box[k] = hd.phys_dim[k];
        q->l = hd.l;
        q->a = hd.a;
        q->tol = hd.tol;
    }
    return h->E.inject(p.size(), p.data(), d.data(), nullptr);
}

nf_status nf_write_coo(nf_handle* h, const char* dir) {
    if (!h || !dir) return NF_ERR_PARAM;
    NF_SINGLE(h, "nf_write_coo");
    nf::Engine& E = h->E;
    if (!E.contacts_valid) return fail(h, NF_ERR_STATE, "no contacts");
    size_t n = E.ct_off[1] - E.ct_off[0];
    std::vector<uint32_t> I(n), J(n);
    std::vector<double> D(n), S(n);
    nf_contact_list c{};
    c.capacity = n;
    c.I = I.data(); c.J = J.data(); c.D = D.data(); c.S = S.data();
    nf_status s = nf_get_contacts(h, &c);
    if (s != NF_OK) return s;
    // save_coo (src/conductivity.cu:838-879): internal, sink, source.
    const char* names[3] = {"internal.srt.coo", "sink.elec.coo", "source.elec.coo"};
    size_t b[4] = {0, E.ct_int[0], E.ct_int[0] + E.ct_snk[0], n};
    for (int f = 0; f < 3; ++f) {
        std::string p = std::string(dir) + "/" + names[f];
        std::ofstream o(p);
        if (!o.is_open()) return NF_ERR_IO;
        o << "#\tI\tJ\tD\tS\n";
        for (size_t q = b[f]; q < b[f + 1]; ++q)
            o << "\t" << I[q] << "\t" << J[q] << "\t" << (float)D[q] << "\t" << (float)S[q] << "\n";
        if (!o.good()) return NF_ERR_IO;
    }
    return NF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Candidate dump without allocation (nf_stream_candidates_noalloc; no
// reference counterpart). The allocating dump stages its output in a device
// buffer it allocates and frees per call; this variant stages it in one fixed
// device array of this translation unit and takes the realisation descriptor
// as a kernel argument, so the call itself allocates no device or host memory.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoAllocMax = NF_NOALLOC_MAX_CANDIDATES;

// Field-major staging: field f of candidate i at [f * kNoAllocMax + i]
// (10 fields x 65536 candidates x 4 B = 2.5 MiB). Nothing here needs to start
// at zero: a call writes all 10 * n values before it copies them out.
static __device__ __align__(256) float g_noalloc_stage[10 * kNoAllocMax];

__global__ void k_stream_dump_static(const nf::Real Re, uint64_t k0, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p, d;
    float u, rho;
    nf::candidate(Re, k0 + i, &p, &d, &u, &rho);
    const float v[10] = {p.x, p.y, p.z, d.x, d.y, d.z, p.w, d.w, u, rho};
    for (int f = 0; f < 10; ++f) out[(size_t)f * kNoAllocMax + i] = v[f];
}

}  // namespace

extern "C" nf_status nf_stream_candidates_noalloc(nf_handle* h, uint64_t k0, uint64_t n, float* x, float* y, float* z,
                                                  float* cx, float* cy, float* cz, float* l, float* a, float* u,
                                                  float* rho) {
    if (!h) return NF_ERR_PARAM;
    nf::Engine& E = h->E;
    if (n > kNoAllocMax)
        return fail(h, NF_ERR_CAPACITY, "nf_stream_candidates_noalloc: n exceeds the fixed staging array of "
                                        "NF_NOALLOC_MAX_CANDIDATES = 65536 candidates");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return E.cuda_fail(e, "cudaGetDevice");
    if (dev != E.dev) return fail(h, NF_ERR_STATE, "nf_stream_candidates_noalloc: current device is not the handle's");
    // The array's device address, looked up on every call with the handle's
    // device current (a host-side query once the module is loaded): an
    // address kept from an earlier call would be stale after a device reset.
    void* addr = nullptr;
    e = cudaGetSymbolAddress(&addr, g_noalloc_stage);
    if (e != cudaSuccess) return E.cuda_fail(e, "cudaGetSymbolAddress(staging array)");
    float* stage = static_cast<float*>(addr);
    // Same descriptor as the allocating dump builds for realisation 0.
    const nf_params& p = E.prm[0];
    const float* dmesh = nullptr;
    if (!E.hmesh[0].empty()) {
        if (E.mesh_dirty || E.hreal.empty())
            return fail(h, NF_ERR_STATE, "nf_stream_candidates_noalloc: the density mesh is not on the device yet "
                                         "(nf_generate or nf_stream_candidates uploads it)");
        dmesh = E.hreal[0].mesh;
    }
    int mn[3] = {p.mesh_ext[0], p.mesh_ext[1], p.mesh_ext[2]};
    const nf::Real Re = nf::make_real(p, dmesh, mn, nf::stage_reach(p));
    if (n) {
        NF_LAUNCH(k_stream_dump_static, (unsigned)((n + 255) / 256), 256, 0, E.st)(Re, k0, (uint32_t)n, stage);
        e = cudaGetLastError();
        if (e != cudaSuccess) return E.cuda_fail(e, "k_stream_dump_static");
    }
    float* dst[10] = {x, y, z, cx, cy, cz, l, a, u, rho};
    for (int f = 0; f < 10 && n; ++f) {
        if (!dst[f]) continue;
        e = cudaMemcpyAsync(dst[f], stage + (size_t)f * kNoAllocMax, sizeof(float) * n, cudaMemcpyDeviceToHost, E.st);
        if (e != cudaSuccess) return E.cuda_fail(e, "nf_stream_candidates_noalloc copy-out");
    }
    e = cudaStreamSynchronize(E.st);
    if (e != cudaSuccess) return E.cuda_fail(e, "nf_stream_candidates_noalloc");
    return NF_OK;
}
