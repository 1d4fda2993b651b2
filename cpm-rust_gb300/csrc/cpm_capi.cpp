// extern "C" surface of libcpm_gpu.so (declared in include/cpm_gpu.h).
//
// The builder restates crates/cpm-py/src/builder.rs:35-525 in C++: string
// parsing with the reference's messages, field-by-field accumulation of the
// user configuration, resolve at run time (config.rs:200-257) and the
// theta helpers. Results wrap cpmhost::Result (convert.rs:27-256).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cpm_gpu.h"
#include "cpm_engine.h"
#include "cpm_host.h"
#include "cpm_kernels.h"
#include "cpm_serve.h"

using namespace cpmhost;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
static int ok() { return CPM_OK; }

extern "C" const char* cpm_last_error(void) { return g_err.c_str(); }
void cpmhost::set_last_error(const std::string& m) { g_err = m; }
extern "C" const char* cpm_version(void) { return "0.2.0+gb300"; }

// Rust's `{:?}` of a &str.
static std::string dbg(const char* s) {
    std::string o = "\"";
    for (const unsigned char* p = (const unsigned char*)s; *p; ++p) {
        const unsigned char c = *p;
        if (c == '"') o += "\\\"";
        else if (c == '\\') o += "\\\\";
        else if (c == '\n') o += "\\n";
        else if (c == '\r') o += "\\r";
        else if (c == '\t') o += "\\t";
        else if (c < 0x20 || c == 0x7f) { char b[16]; std::snprintf(b, sizeof b, "\\u{%x}", c); o += b; }
        else o += (char)c;
    }
    return o + "\"";
}

struct cpm_builder {
    Config cfg;  // grid, boundary, seed and neighbourhoods are set at construction
    bool energy_set = false;
    bool adhesion_set = false;
    bool init_set = false;
    std::map<std::string, size_t> type_index;
};

struct cpm_result {
    Result r;
};

// builder.rs:35-96
static int parse_boundary(const char* s, bool& periodic) {
    if (!std::strcmp(s, "fixed")) { periodic = false; return 0; }
    if (!std::strcmp(s, "periodic")) { periodic = true; return 0; }
    return fail(CPM_E_CONFIG, "unknown boundary " + dbg(s) + "; expected \"fixed\" or \"periodic\"");
}
static int parse_nbh(const char* s, int& k) {
    static const char* names[] = {"von_neumann", "moore", "eighteen", "twenty_six", "twenty_six_weighted"};
    for (int i = 0; i < 5; ++i)
        if (!std::strcmp(s, names[i])) { k = i; return 0; }
    return fail(CPM_E_CONFIG, "unknown neighbourhood " + dbg(s) +
                                  "; expected one of \"von_neumann\", \"moore\", \"eighteen\", \"twenty_six\", "
                                  "\"twenty_six_weighted\"");
}

extern "C" int cpm_builder_new(const uint64_t* grid, size_t grid_len, const char* boundary, uint64_t seed,
                               const char* copy_neighborhood, const char* energy_neighborhood,
                               const char* connectivity_neighborhood, const char* acceptance, const char* proposal,
                               const char* const* keys, const int32_t* values, size_t n_keys, cpm_builder** out) {
    if (!out || !boundary || !copy_neighborhood || !connectivity_neighborhood || (grid_len && !grid) ||
        (n_keys && (!keys || !values)))
        return fail(CPM_E_ARG, "null argument");
    auto b = std::make_unique<cpm_builder>();
    int e;
    if ((e = parse_boundary(boundary, b->cfg.periodic))) return e;
    if ((e = parse_nbh(copy_neighborhood, b->cfg.copy_nbh))) return e;
    if (energy_neighborhood) {
        if ((e = parse_nbh(energy_neighborhood, b->cfg.energy_nbh))) return e;
        b->energy_set = true;
    }
    if ((e = parse_nbh(connectivity_neighborhood, b->cfg.conn_nbh))) return e;
    if (acceptance) {
        if (!std::strcmp(acceptance, "metropolis")) b->cfg.acceptance = ACC_METROPOLIS;
        else if (!std::strcmp(acceptance, "metropolis_hastings")) b->cfg.acceptance = ACC_METROPOLIS_HASTINGS;
        else return fail(CPM_E_CONFIG, "unknown acceptance mode " + dbg(acceptance) +
                                           "; expected \"metropolis\" or \"metropolis_hastings\"");
    }
    if (proposal) {
        if (!std::strcmp(proposal, "uniform")) b->cfg.proposal = PROP_UNIFORM;
        else if (!std::strcmp(proposal, "edge_list")) b->cfg.proposal = PROP_EDGE_LIST;
        else return fail(CPM_E_CONFIG, "unknown proposal mode " + dbg(proposal) + "; expected \"uniform\" or \"edge_list\"");
    }
    for (size_t i = 0; i < n_keys; ++i) {
        if (!keys[i]) return fail(CPM_E_ARG, "null argument");
        const bool v = values[i] != 0;
        if (!std::strcmp(keys[i], "volume")) b->cfg.active.volume = v;
        else if (!std::strcmp(keys[i], "interface")) b->cfg.active.interface = v;
        else if (!std::strcmp(keys[i], "adhesion")) b->cfg.active.adhesion = v;
        else if (!std::strcmp(keys[i], "act")) b->cfg.active.act = v;
        else return fail(CPM_E_CONFIG, "unknown active_terms key " + dbg(keys[i]) +
                                           "; expected one of \"volume\", \"interface\", \"adhesion\", \"act\"");
    }
    if (grid_len != 2 && grid_len != 3)
        return fail(CPM_E_CONFIG, "grid must have length 2 or 3 (dimensionality is inferred from it, not from an "
                                  "explicit `dimension` argument); got length " + std::to_string(grid_len));
    b->cfg.D = (int)grid_len;
    for (size_t d = 0; d < grid_len; ++d) b->cfg.grid[d] = (int64_t)grid[d];
    b->cfg.seed = seed;
    *out = b.release();
    return ok();
}

extern "C" int cpm_builder_register_cell_type(cpm_builder* b, const char* name, uint32_t target_volume,
                                              uint32_t target_interface, double lambda_volume, double lambda_interface,
                                              double lambda_act, uint32_t max_act) {
    if (!b || !name) return fail(CPM_E_ARG, "null argument");
    if (b->type_index.count(name)) return fail(CPM_E_CONFIG, "cell type " + dbg(name) + " has already been added");
    CellType t;
    t.name = name;
    t.target_volume = target_volume;
    t.target_interface = target_interface;
    t.lambda_volume = lambda_volume;
    t.lambda_interface = lambda_interface;
    t.lambda_act = lambda_act;
    t.max_act = max_act;
    const std::string e = cell_type_error(t);
    if (!e.empty()) return fail(CPM_E_CONFIG, e);
    const size_t idx = b->type_index.size();
    b->type_index[name] = idx;
    b->cfg.types.push_back(t);
    b->cfg.cell_counts.push_back(0);
    return ok();
}

extern "C" int cpm_builder_add_cells(cpm_builder* b, const char* cell_type, uint64_t n) {
    if (!b || !cell_type) return fail(CPM_E_ARG, "null argument");
    auto it = b->type_index.find(cell_type);
    if (it == b->type_index.end())
        return fail(CPM_E_CONFIG, "unknown cell type " + dbg(cell_type) + "; call register_cell_type first");
    b->cfg.cell_counts[it->second] = n;
    return ok();
}

extern "C" int cpm_builder_set_adhesion(cpm_builder* b, const double* values, const size_t* row_lengths, size_t n_rows) {
    if (!b || (n_rows && (!row_lengths))) return fail(CPM_E_ARG, "null argument");
    size_t total = 0;
    for (size_t r = 0; r < n_rows; ++r) total += row_lengths[r];
    if (total && !values) return fail(CPM_E_ARG, "null argument");
    b->cfg.adhesion.assign(n_rows, {});
    size_t k = 0;
    for (size_t r = 0; r < n_rows; ++r) {
        b->cfg.adhesion[r].assign(values + k, values + k + row_lengths[r]);
        k += row_lengths[r];
    }
    b->adhesion_set = true;
    return ok();
}

extern "C" int cpm_builder_initialize(cpm_builder* b, const uint32_t* lattice, size_t lattice_len,
                                      const uint64_t* cell_type_of, size_t cto_len, int32_t has_cto, int32_t warn) {
    if (!b) return fail(CPM_E_ARG, "null argument");
    if (lattice) {
        if (!has_cto) return fail(CPM_E_CONFIG, "cell_type_of is required when lattice is supplied");
        if (cto_len && !cell_type_of) return fail(CPM_E_ARG, "null argument");
        b->cfg.init_explicit = true;
        b->cfg.init_lattice.assign(lattice, lattice + lattice_len);
        b->cfg.init_type_of.assign(cell_type_of, cell_type_of + cto_len);
    } else {
        b->cfg.init_explicit = false;
        b->cfg.init_lattice.clear();
        b->cfg.init_type_of.clear();
        b->cfg.warn_on_default_init = warn != 0;
    }
    b->init_set = true;
    return ok();
}

// UserConfig::resolve (config.rs:200-257) with the windows supplied.
static int resolve(const cpm_builder* b, uint64_t burn, uint64_t readout, uint64_t interval, Config& c) {
    if (!b->adhesion_set) return fail(CPM_E_CONFIG, "adhesion matrix is required");
    c = b->cfg;
    if (!b->energy_set) c.energy_nbh = c.D == 2 ? NBH_MOORE : NBH_EIGHTEEN;
    c.burn_in = burn;
    c.readout = readout;
    c.interval = interval;
    c.min_cell_volume = 1;
    return ok();
}

// Every configuration the reference accepts runs here. The EdgeList
// proposal (monte_carlo.rs:336-352) is, by the reference's own definition
// (edge_list.rs:1-16), the Uniform chain with its null attempts removed; the
// device sweep visits every site and a null attempt costs it one
// comparison, so both proposals run the same device chain (the convention
// hash still records which one was asked for).

static int code_for(const std::string& e) {
    if (e.rfind("CUDA error", 0) == 0) return CPM_E_CUDA;
    if (e.find("timed out") != std::string::npos) return CPM_E_TIMEOUT;
    return CPM_E_INIT;
}

extern "C" int cpm_builder_run(const cpm_builder* b, uint64_t burn, uint64_t readout, uint64_t interval,
                               int32_t include_lattice, int32_t* used_default, cpm_result** out) {
    if (!b || !out) return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve(b, burn, readout, interval, c);
    if (e) return e;
    std::string msg = validate(c);
    if (!msg.empty()) return fail(CPM_E_CONFIG, msg);
    Initial init;
    const auto t0 = std::chrono::steady_clock::now();
    msg = initialize(c, init);
    if (!msg.empty()) return fail(CPM_E_INIT, msg);
    const uint64_t place_us =
        (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
    ReadoutOptions ro;
    ro.include_lattice = include_lattice != 0;
    ro.topology = true;
    std::vector<Result> rs;
    msg = run_many({c}, {init}, ro, rs);
    if (!msg.empty()) return fail(code_for(msg), msg);
    if (rs[0].stats.size() > CPM_STAT_HOST_PLACE_US) rs[0].stats[CPM_STAT_HOST_PLACE_US] = place_us;
    auto r = std::make_unique<cpm_result>();
    r->r = std::move(rs[0]);
    if (used_default) *used_default = init.used_default;
    *out = r.release();
    return ok();
}

extern "C" int cpm_builder_run_batch(const cpm_builder* b, const double* thetas, const size_t* lens, size_t n,
                                     uint64_t burn, uint64_t readout, uint64_t interval, uint64_t master_seed,
                                     int32_t include_lattice, int32_t* any_used_default, cpm_result** out) {
    if (!b || (n && (!out || !lens))) return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve(b, burn, readout, interval, c);
    if (e) return e;
    const size_t expected = theta_len(c.types.size());
    if (n && expected && !thetas) return fail(CPM_E_ARG, "null argument");
    std::vector<std::vector<double>> th(n);
    size_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        if (lens[i] != expected)
            return fail(CPM_E_THETA, "theta at index " + std::to_string(i) + " has length " + std::to_string(lens[i]) +
                                         ", expected " + std::to_string(expected));
        th[i].assign(thetas + k, thetas + k + lens[i]);
        k += lens[i];
    }
    ReadoutOptions ro;
    ro.include_lattice = include_lattice != 0;
    ro.topology = true;
    std::vector<Result> rs;
    BatchStage stage = BATCH_OK;
    const std::string msg = run_batch(c, th, master_seed, ro, rs, &stage);
    if (!msg.empty()) {
        const int code = stage == BATCH_THETA    ? CPM_E_THETA
                         : stage == BATCH_CONFIG ? CPM_E_CONFIG
                         : stage == BATCH_INIT   ? CPM_E_INIT
                                                 : code_for(msg);
        return fail(code, msg);
    }
    bool any = false;
    for (size_t i = 0; i < n; ++i) {
        any = any || rs[i].used_default;
        auto r = std::make_unique<cpm_result>();
        r->r = std::move(rs[i]);
        out[i] = r.release();
    }
    if (any_used_default) *any_used_default = any;
    return ok();
}

// builder.rs:405-430: placeholder windows, then resolve + validate.
static int resolve_for_theta(const cpm_builder* b, Config& c) {
    int e = resolve(b, 1, 1, 1, c);
    if (e) return e;
    const std::string msg = validate(c);
    if (!msg.empty()) return fail(CPM_E_CONFIG, msg);
    return ok();
}

extern "C" int cpm_builder_theta_len(const cpm_builder* b, size_t* out) {
    if (!b || !out) return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve_for_theta(b, c);
    if (e) return e;
    *out = theta_len(c.types.size());
    return ok();
}

extern "C" int cpm_builder_extract_theta(const cpm_builder* b, double* out, size_t cap) {
    if (!b || !out) return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve_for_theta(b, c);
    if (e) return e;
    const std::vector<double> th = theta_extract(c);
    if (cap < th.size()) return fail(CPM_E_ARG, "buffer too small");
    std::memcpy(out, th.data(), th.size() * sizeof(double));
    return ok();
}

extern "C" int cpm_builder_theta_name(const cpm_builder* b, size_t index, char* buf, size_t cap) {
    if (!b || !buf) return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve_for_theta(b, c);
    if (e) return e;
    const std::vector<std::string> names = theta_names(c);
    if (index >= names.size()) return fail(CPM_E_ARG, "theta index out of range");
    if (cap < names[index].size() + 1) return fail(CPM_E_ARG, "buffer too small");
    std::memcpy(buf, names[index].c_str(), names[index].size() + 1);
    return ok();
}

extern "C" void cpm_builder_free(cpm_builder* b) { delete b; }

// ------------------------------------------------------------- results ----
extern "C" int cpm_result_info_get(const cpm_result* r, cpm_result_info* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    std::memset(o, 0, sizeof *o);
    o->dim = r->r.D;
    o->n_types = (int32_t)r->r.cell_type_names.size();
    for (size_t d = 0; d < r->r.grid.size(); ++d) o->grid[d] = r->r.grid[d];
    o->n_cells = r->r.cell_type_index.size();
    o->n_samples = r->r.samples.size();
    o->used_default = r->r.used_default;
    return ok();
}

static void copy_str(char* dst, size_t cap, const std::string& s) {
    std::snprintf(dst, cap, "%s", s.c_str());
}

extern "C" int cpm_result_metadata_get(const cpm_result* r, cpm_metadata* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    std::memset(o, 0, sizeof *o);
    const Metadata& m = r->r.metadata;
    copy_str(o->cpm_version, sizeof o->cpm_version, m.cpm_version);
    copy_str(o->convention_hash, sizeof o->convention_hash, m.convention_hash);
    copy_str(o->model_hash, sizeof o->model_hash, m.model_hash);
    copy_str(o->seed_policy, sizeof o->seed_policy, m.seed_policy);
    o->convention_version = m.convention_version;
    o->theta_layout_version = m.theta_layout_version;
    o->seed = m.seed;
    o->derived_phi = m.derived_phi;
    return ok();
}

extern "C" int cpm_result_status_get(const cpm_result* r, cpm_status* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    std::memset(o, 0, sizeof *o);
    copy_str(o->kind, sizeof o->kind, r->r.status.kind);
    o->has_cell = r->r.status.has_cell;
    o->cell_id = r->r.status.cell_id;
    o->at_mcs = r->r.status.at_mcs;
    return ok();
}

extern "C" int cpm_result_cell_type_index(const cpm_result* r, uint32_t* out) {
    if (!r || !out) return fail(CPM_E_ARG, "null argument");
    std::memcpy(out, r->r.cell_type_index.data(), r->r.cell_type_index.size() * 4);
    return ok();
}

extern "C" int cpm_result_cell_type_name(const cpm_result* r, size_t t, char* buf, size_t cap) {
    if (!r || !buf) return fail(CPM_E_ARG, "null argument");
    if (t >= r->r.cell_type_names.size()) return fail(CPM_E_ARG, "type index out of range");
    const std::string& s = r->r.cell_type_names[t];
    if (cap < s.size() + 1) return fail(CPM_E_ARG, "buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return ok();
}

extern "C" int cpm_result_sample_sizes(const cpm_result* r, size_t s, cpm_sample_sizes* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    if (s >= r->r.samples.size()) return fail(CPM_E_ARG, "sample index out of range");
    const Sample& S = r->r.samples[s];
    std::memset(o, 0, sizeof *o);
    o->n_contact = S.contact_a.size();
    o->n_fragmented = S.fragmented.size();
    o->n_medium = S.medium_volumes.size();
    o->has_lattice = S.has_lattice;
    return ok();
}

extern "C" int cpm_result_sample_read(const cpm_result* r, size_t s, const cpm_sample_out* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    if (s >= r->r.samples.size()) return fail(CPM_E_ARG, "sample index out of range");
    const Sample& S = r->r.samples[s];
    const int D = r->r.D;
    if (o->mcs) *o->mcs = S.mcs;
    if (o->conservative_energy) *o->conservative_energy = S.energy;
    for (size_t i = 0; i < S.cells.size(); ++i) {
        const CellSample& c = S.cells[i];
        if (o->ids) o->ids[i] = c.id;
        if (o->volume) o->volume[i] = c.volume;
        if (o->interface) o->interface[i] = c.interface;
        for (int d = 0; d < D; ++d) {
            if (o->centroid) o->centroid[i * D + d] = c.centroid[d];
            if (o->eigenvalues) o->eigenvalues[i * D + d] = c.eigenvalues[d];
        }
        if (o->radius_of_gyration_sq) o->radius_of_gyration_sq[i] = c.rg2;
        if (o->kappa_sq) o->kappa_sq[i] = c.kappa2;
    }
    for (size_t k = 0; k < S.contact_a.size(); ++k) {
        if (o->contact_a) o->contact_a[k] = S.contact_a[k];
        if (o->contact_b) o->contact_b[k] = S.contact_b[k];
        if (o->contact_count) o->contact_count[k] = S.contact_n[k];
    }
    if (o->fragmented_cells && !S.fragmented.empty())
        std::memcpy(o->fragmented_cells, S.fragmented.data(), S.fragmented.size() * 4);
    if (o->medium_component_volumes && !S.medium_volumes.empty())
        std::memcpy(o->medium_component_volumes, S.medium_volumes.data(), S.medium_volumes.size() * 4);
    if (o->medium_component_touches_boundary && !S.medium_touches.empty())
        std::memcpy(o->medium_component_touches_boundary, S.medium_touches.data(), S.medium_touches.size());
    if (o->lattice && S.has_lattice) std::memcpy(o->lattice, S.lattice.data(), S.lattice.size() * 4);
    return ok();
}

extern "C" int cpm_result_samples_sizes(const cpm_result* r, cpm_samples_sizes* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    std::memset(o, 0, sizeof *o);
    o->n_samples = r->r.samples.size();
    o->n_cells = r->r.cell_type_index.size();
    for (const Sample& S : r->r.samples) {
        o->total_contact += S.contact_a.size();
        o->total_fragmented += S.fragmented.size();
        o->total_medium += S.medium_volumes.size();
        o->has_lattice |= S.has_lattice ? 1 : 0;
    }
    return ok();
}

static void samples_read(const cpm_result* r, const cpm_samples_out* o) {
    const int D = r->r.D;
    const size_t n = r->r.cell_type_index.size();
    size_t nc = 0, nf = 0, nm = 0, site0 = 0;
    for (size_t s = 0; s < r->r.samples.size(); ++s) {
        const Sample& S = r->r.samples[s];
        if (o->mcs) o->mcs[s] = S.mcs;
        if (o->conservative_energy) o->conservative_energy[s] = S.energy;
        for (size_t i = 0; i < S.cells.size() && i < n; ++i) {
            const CellSample& c = S.cells[i];
            const size_t k = s * n + i;
            if (o->ids) o->ids[k] = c.id;
            if (o->volume) o->volume[k] = c.volume;
            if (o->interface) o->interface[k] = c.interface;
            for (int d = 0; d < D; ++d) {
                if (o->centroid) o->centroid[k * D + d] = c.centroid[d];
                if (o->eigenvalues) o->eigenvalues[k * D + d] = c.eigenvalues[d];
            }
            if (o->radius_of_gyration_sq) o->radius_of_gyration_sq[k] = c.rg2;
            if (o->kappa_sq) o->kappa_sq[k] = c.kappa2;
        }
        if (o->contact_offsets) o->contact_offsets[s] = nc;
        for (size_t k = 0; k < S.contact_a.size(); ++k, ++nc) {
            if (o->contact_a) o->contact_a[nc] = S.contact_a[k];
            if (o->contact_b) o->contact_b[nc] = S.contact_b[k];
            if (o->contact_count) o->contact_count[nc] = S.contact_n[k];
        }
        if (o->fragmented_offsets) o->fragmented_offsets[s] = nf;
        if (o->fragmented_cells && !S.fragmented.empty())
            std::memcpy(o->fragmented_cells + nf, S.fragmented.data(), S.fragmented.size() * 4);
        nf += S.fragmented.size();
        if (o->medium_offsets) o->medium_offsets[s] = nm;
        if (o->medium_component_volumes && !S.medium_volumes.empty())
            std::memcpy(o->medium_component_volumes + nm, S.medium_volumes.data(), S.medium_volumes.size() * 4);
        if (o->medium_component_touches_boundary && !S.medium_touches.empty())
            std::memcpy(o->medium_component_touches_boundary + nm, S.medium_touches.data(), S.medium_touches.size());
        nm += S.medium_volumes.size();
        if (o->lattice && S.has_lattice) {
            std::memcpy(o->lattice + site0, S.lattice.data(), S.lattice.size() * 4);
            site0 += S.lattice.size();
        }
    }
    const size_t ns = r->r.samples.size();
    if (o->contact_offsets) o->contact_offsets[ns] = nc;
    if (o->fragmented_offsets) o->fragmented_offsets[ns] = nf;
    if (o->medium_offsets) o->medium_offsets[ns] = nm;
}

extern "C" int cpm_result_samples_read(const cpm_result* r, const cpm_samples_out* o) {
    if (!r || !o) return fail(CPM_E_ARG, "null argument");
    samples_read(r, o);
    return ok();
}

extern "C" int cpm_results_samples_read(const cpm_result* const* rs, size_t n, const cpm_samples_out* outs) {
    if (n && (!rs || !outs)) return fail(CPM_E_ARG, "null argument");
    for (size_t i = 0; i < n; ++i)
        if (!rs[i]) return fail(CPM_E_ARG, "null result");
    std::atomic<size_t> next{0};
    auto work = [&] {
        for (size_t i; (i = next.fetch_add(1)) < n;) samples_read(rs[i], &outs[i]);
    };
    const size_t nt = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), (n + 7) / 8);
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; ++t) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    return ok();
}

extern "C" int cpm_result_stats(const cpm_result* r, uint64_t* out32) {
    if (!r || !out32) return fail(CPM_E_ARG, "null argument");
    std::memset(out32, 0, 32 * sizeof(uint64_t));
    for (size_t i = 0; i < r->r.stats.size() && i < 32; ++i) out32[i] = r->r.stats[i];
    return ok();
}

extern "C" void cpm_result_free(cpm_result* r) { delete r; }

// -------------------------------------------------------------- engine ----
struct cpm_engine {
    std::vector<Config> configs;
    std::vector<Initial> initials;
    DeviceSims sims;
    double* d_energy = nullptr;
    uint32_t* d_recount = nullptr;
    size_t recount_cap = 0;
    ~cpm_engine() {
        if (d_energy) cudaFree(d_energy);
        if (d_recount) cudaFree(d_recount);
    }
};

static int prepare(const cpm_builder* const* builders, size_t n, std::vector<Config>& cfgs, std::vector<Initial>& inits,
                   uint64_t burn, uint64_t readout, uint64_t interval) {
    cfgs.resize(n);
    inits.resize(n);
    for (size_t i = 0; i < n; ++i) {
        if (!builders[i]) return fail(CPM_E_ARG, "null builder");
        int e = resolve(builders[i], burn, readout, interval, cfgs[i]);
        if (e) return e;
        std::string msg = validate(cfgs[i]);
        if (!msg.empty()) return fail(CPM_E_CONFIG, msg);
    }
    // placements are independent: host threads over simulations; the first
    // failure in input order is reported
    std::vector<std::string> errs(n);
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < n;) errs[i] = initialize(cfgs[i], inits[i]);
    };
    const unsigned nthreads = (unsigned)std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), n));
    if (nthreads == 1) {
        worker();
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nthreads; ++t) th.emplace_back(worker);
        for (auto& t : th) t.join();
    }
    for (size_t i = 0; i < n; ++i)
        if (!errs[i].empty()) return fail(CPM_E_INIT, errs[i]);
    return ok();
}

extern "C" int cpm_engine_create(const cpm_builder* const* builders, size_t n, void* stream, cpm_engine** out) {
    if (!builders || !out || n == 0) return fail(CPM_E_ARG, "null argument");
    auto e = std::make_unique<cpm_engine>();
    int rc = prepare(builders, n, e->configs, e->initials, 1, 1, 1);
    if (rc) return rc;
    std::vector<int> ones(n, 1);  // one sample slot (with its lattice) for cpm_engine_take_sample
    const std::string msg = e->sims.create(e->configs, e->initials, ones, ones, true, (cudaStream_t)stream);
    if (!msg.empty()) return fail(code_for(msg), msg);
    if (cudaMalloc(&e->d_energy, sizeof(double)) != cudaSuccess) return fail(CPM_E_CUDA, "cudaMalloc failed");
    *out = e.release();
    return ok();
}

extern "C" int cpm_engine_size(const cpm_engine* e, size_t* out) {
    if (!e || !out) return fail(CPM_E_ARG, "null argument");
    *out = e->sims.size();
    return ok();
}

static bool bad_sim(const cpm_engine* e, size_t i) { return !e || i >= e->sims.size(); }

extern "C" int cpm_engine_sim_info(const cpm_engine* e, size_t i, cpm_sim_info* o) {
    if (bad_sim(e, i) || !o) return fail(CPM_E_ARG, "bad engine or simulation index");
    const SimLayout& L = e->sims.layout(i);
    const SimDesc& s = e->sims.host_desc(i);
    std::memset(o, 0, sizeof *o);
    o->dim = L.g.D;
    o->periodic = L.g.periodic;
    for (int d = 0; d < 3; ++d) { o->dims[d] = L.g.dims[d]; o->padded_dims[d] = L.g.pdims[d]; o->strides[d] = L.g.strides[d]; }
    o->n_sites = L.g.n_sites;
    o->n_padded = L.g.n_padded;
    o->n_cells = L.n_cells;
    o->n_energy = L.NE;
    o->n_colors = s.n_colors;
    return ok();
}

extern "C" int cpm_engine_run_mcs(cpm_engine* e, uint64_t n) {
    if (!e) return fail(CPM_E_ARG, "null argument");
    if (n == 0) return ok();
    std::vector<RunPlan> plans(e->sims.size());
    for (size_t i = 0; i < plans.size(); ++i) {
        RunPlan& p = plans[i];
        std::memset(&p, 0, sizeof p);
        p.sim = (int)i;
        p.burn_in = n;
        p.interval = n;
        p.energy_sample_start = ~0ull;
        p.n_samples = 0;
    }
    const std::string msg = e->sims.run(plans);
    if (!msg.empty()) return fail(code_for(msg), msg);
    return ok();
}

extern "C" int cpm_engine_take_sample(cpm_engine* e, size_t i, int32_t include_lattice, cpm_result** out) {
    if (bad_sim(e, i) || !out) return fail(CPM_E_ARG, "bad engine or simulation index");
    DeviceSims& S = e->sims;
    const SimLayout& L = S.layout(i);
    cudaError_t ce = cpmgpu::launch_sample(L.g.D, S.device_desc(i), 0, 1, L.g.n_sites, S.stream());
    if (ce == cudaSuccess)
        ce = cpmgpu::launch_energy(L.g.D, L.NE, S.device_desc(i), S.host_desc(i).energy_out, S.stream());
    if (ce != cudaSuccess) return fail(CPM_E_CUDA, std::string("CUDA error: ") + cudaGetErrorString(ce));
    std::vector<std::vector<Topo>> topo;
    std::string msg = S.topology({i}, {1}, topo);
    if (msg.empty()) msg = S.sync();
    ReadoutOptions ro;
    ro.include_lattice = include_lattice != 0;
    ro.topology = true;
    Result R;
    if (msg.empty()) msg = assemble_result(e->configs[i], e->initials[i], S, i, 1, 0, ro, R);
    uint64_t mcs = 0;
    if (msg.empty()) msg = S.read_mcs(i, mcs);
    if (!msg.empty()) return fail(code_for(msg), msg);
    R.samples[0].mcs = mcs;
    attach_topology(e->configs[i], topo[0], R);
    auto r = std::make_unique<cpm_result>();
    r->r = std::move(R);
    *out = r.release();
    return ok();
}

extern "C" int cpm_engine_write_act_state(cpm_engine* e, size_t i, const uint32_t* birth, uint64_t mcs) {
    if (bad_sim(e, i)) return fail(CPM_E_ARG, "bad engine or simulation index");
    std::vector<uint32_t> b;
    if (birth) b.assign(birth, birth + e->sims.layout(i).g.n_padded);
    const std::string msg = e->sims.write_act_state(i, birth ? &b : nullptr, mcs);
    return msg.empty() ? ok() : fail(msg.rfind("CUDA", 0) == 0 ? CPM_E_CUDA : CPM_E_ARG, msg);
}

extern "C" int cpm_engine_read_birth(const cpm_engine* e, size_t i, uint32_t* out) {
    if (bad_sim(e, i) || !out) return fail(CPM_E_ARG, "bad engine or simulation index");
    std::vector<uint32_t> b;
    const std::string msg = e->sims.read_birth(i, b);
    if (!msg.empty()) return fail(msg.rfind("CUDA", 0) == 0 ? CPM_E_CUDA : CPM_E_ARG, msg);
    std::memcpy(out, b.data(), b.size() * 4);
    return ok();
}

extern "C" int cpm_engine_synchronize(cpm_engine* e) {
    if (!e) return fail(CPM_E_ARG, "null argument");
    const std::string msg = e->sims.sync();
    if (!msg.empty()) return fail(code_for(msg) == CPM_E_TIMEOUT ? CPM_E_TIMEOUT : CPM_E_CUDA, msg);
    return ok();
}

extern "C" int cpm_engine_mcs(const cpm_engine* e, size_t i, uint64_t* out) {
    if (bad_sim(e, i) || !out) return fail(CPM_E_ARG, "bad engine or simulation index");
    const std::string msg = e->sims.read_mcs(i, *out);
    return msg.empty() ? ok() : fail(CPM_E_CUDA, msg);
}

extern "C" int cpm_engine_read_padded(const cpm_engine* e, size_t i, uint32_t* out) {
    if (bad_sim(e, i) || !out) return fail(CPM_E_ARG, "bad engine or simulation index");
    std::vector<uint32_t> p;
    const std::string msg = e->sims.read_padded(i, p);
    if (!msg.empty()) return fail(CPM_E_CUDA, msg);
    std::memcpy(out, p.data(), p.size() * 4);
    return ok();
}

extern "C" int cpm_engine_read_lattice(const cpm_engine* e, size_t i, uint32_t* out) {
    if (bad_sim(e, i) || !out) return fail(CPM_E_ARG, "bad engine or simulation index");
    std::vector<uint32_t> p;
    const std::string msg = e->sims.read_padded(i, p);
    if (!msg.empty()) return fail(CPM_E_CUDA, msg);
    const Geometry& g = e->sims.layout(i).g;
    int64_t x[3] = {0, 0, 0};
    for (int64_t q = 0; q < g.n_sites; ++q) {
        out[q] = p[g.flat(x)];
        for (int d = g.D - 1; d >= 0; --d) { if (++x[d] < g.dims[d]) break; x[d] = 0; }
    }
    return ok();
}

extern "C" int cpm_engine_read_cells(const cpm_engine* e, size_t i, uint32_t* volume, uint32_t* interface,
                                     int64_t* sp, int64_t* so) {
    if (bad_sim(e, i)) return fail(CPM_E_ARG, "bad engine or simulation index");
    std::vector<uint32_t> v, it;
    std::vector<int64_t> a, b;
    const std::string msg = e->sims.read_cells(i, v, it, a, b);
    if (!msg.empty()) return fail(CPM_E_CUDA, msg);
    if (volume) std::memcpy(volume, v.data(), v.size() * 4);
    if (interface) std::memcpy(interface, it.data(), it.size() * 4);
    if (sp) std::memcpy(sp, a.data(), a.size() * 8);
    if (so) std::memcpy(so, b.data(), b.size() * 8);
    return ok();
}

extern "C" int cpm_engine_energy(const cpm_engine* e, size_t i, double* out) {
    if (bad_sim(e, i) || !out) return fail(CPM_E_ARG, "bad engine or simulation index");
    const SimLayout& L = e->sims.layout(i);
    cudaError_t ce = cpmgpu::launch_energy(L.g.D, L.NE, e->sims.device_desc(i), e->d_energy, e->sims.stream());
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(out, e->d_energy, sizeof(double), cudaMemcpyDeviceToHost, e->sims.stream());
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->sims.stream());
    if (ce != cudaSuccess) return fail(CPM_E_CUDA, std::string("CUDA error: ") + cudaGetErrorString(ce));
    return ok();
}

extern "C" int cpm_engine_recount_check(const cpm_engine* ec, size_t i, int32_t* okp, uint32_t* volume, uint32_t* interface) {
    cpm_engine* e = const_cast<cpm_engine*>(ec);
    if (bad_sim(e, i)) return fail(CPM_E_ARG, "bad engine or simulation index");
    const SimLayout& L = e->sims.layout(i);
    const size_t n1 = L.n_cells + 1;
    if (e->recount_cap < 2 * n1) {
        if (e->d_recount) cudaFree(e->d_recount);
        e->d_recount = nullptr;
        if (cudaMalloc(&e->d_recount, 2 * n1 * 4) != cudaSuccess) return fail(CPM_E_CUDA, "cudaMalloc failed");
        e->recount_cap = 2 * n1;
    }
    cudaStream_t st = e->sims.stream();
    cudaError_t ce = cudaMemsetAsync(e->d_recount, 0, 2 * n1 * 4, st);
    if (ce == cudaSuccess)
        ce = cpmgpu::launch_recount(L.g.D, L.NE, e->sims.device_desc(i), L.g.n_sites, e->d_recount, e->d_recount + n1, st);
    std::vector<uint32_t> rc(2 * n1);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(rc.data(), e->d_recount, 2 * n1 * 4, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return fail(CPM_E_CUDA, std::string("CUDA error: ") + cudaGetErrorString(ce));
    std::vector<uint32_t> v, it;
    std::vector<int64_t> a, b;
    const std::string msg = e->sims.read_cells(i, v, it, a, b);
    if (!msg.empty()) return fail(CPM_E_CUDA, msg);
    bool same = true;
    for (size_t id = 1; id < n1; ++id)
        if (rc[id] != v[id] || rc[n1 + id] != it[id]) same = false;
    if (okp) *okp = same;
    if (volume) std::memcpy(volume, rc.data(), n1 * 4);
    if (interface) std::memcpy(interface, rc.data() + n1, n1 * 4);
    return ok();
}

extern "C" int cpm_engine_stats(const cpm_engine* e, size_t i, uint64_t* out32) {
    if (bad_sim(e, i) || !out32) return fail(CPM_E_ARG, "bad engine or simulation index");
    std::vector<uint64_t> s;
    const std::string msg = e->sims.read_stats(i, s);
    if (!msg.empty()) return fail(CPM_E_CUDA, msg);
    std::memset(out32, 0, 32 * 8);
    std::memcpy(out32, s.data(), std::min<size_t>(s.size(), 32) * 8);
    return ok();
}

extern "C" int cpm_engine_write_state(cpm_engine* e, size_t i, const uint32_t* padded, const uint32_t* volume,
                                      const uint32_t* interface, const int64_t* sp, const int64_t* so) {
    if (bad_sim(e, i) || !padded || !volume || !interface) return fail(CPM_E_ARG, "bad engine, index or buffer");
    const SimLayout& L = e->sims.layout(i);
    const size_t n1 = L.n_cells + 1, D = L.g.D;
    std::vector<uint32_t> p(padded, padded + L.g.n_padded), v(volume, volume + n1), it(interface, interface + n1);
    std::vector<int64_t> a, b;
    if (sp) a.assign(sp, sp + n1 * D);
    if (so) b.assign(so, so + n1 * D * D);
    const std::string msg = e->sims.write_state(i, p, v, it, sp ? &a : nullptr, so ? &b : nullptr);
    return msg.empty() ? ok() : fail(msg.rfind("CUDA", 0) == 0 ? CPM_E_CUDA : CPM_E_ARG, msg);
}

extern "C" int cpm_engine_evaluate_moves(cpm_engine* e, size_t i, size_t n, const int64_t* target, const int32_t* k,
                                         const double* u, cpm_move* out) {
    if (bad_sim(e, i) || (n && (!target || !k || !u || !out))) return fail(CPM_E_ARG, "bad engine, index or buffer");
    if (n == 0) return ok();
    const SimLayout& L = e->sims.layout(i);
    const int ncopy = 2 * L.g.D;
    for (size_t m = 0; m < n; ++m) {
        if (k[m] < 0 || k[m] >= ncopy) return fail(CPM_E_ARG, "copy direction out of range");
        // the target must be an interior site (its stencil then stays inside the padded array)
        int64_t f = target[m];
        if (f < 0 || f >= L.g.n_padded) return fail(CPM_E_ARG, "target outside the lattice");
        for (int d = 0; d < L.g.D; ++d) {
            const int64_t c = f / L.g.strides[d];
            f %= L.g.strides[d];
            if (c == 0 || c == L.g.pdims[d] - 1) return fail(CPM_E_ARG, "target is a halo site");
        }
    }
    std::string err;
    const uint64_t* t3 = L.g.D == 3 ? device_table3d(err) : nullptr;
    if (L.g.D == 3 && !t3) return fail(CPM_E_CUDA, err);
    int64_t* d_t = nullptr;
    int32_t* d_k = nullptr;
    double* d_u = nullptr;
    MoveOut* d_o = nullptr;
    cudaError_t ce = cudaMalloc(&d_t, n * 8);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_k, n * 4);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_u, n * 8);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_o, n * sizeof(MoveOut));
    cudaStream_t st = e->sims.stream();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_t, target, n * 8, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_k, k, n * 4, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_u, u, n * 8, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cpmgpu::launch_evaluate(L.g.D, L.NE, e->sims.device_desc(i), (int64_t)n, d_t, d_k, d_u, d_o, t3, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(out, d_o, n * sizeof(MoveOut), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    cudaFree(d_t); cudaFree(d_k); cudaFree(d_u); cudaFree(d_o);
    if (ce != cudaSuccess) return fail(CPM_E_CUDA, std::string("CUDA error: ") + cudaGetErrorString(ce));
    return ok();
}

extern "C" int cpm_engine_commit_moves(cpm_engine* e, size_t i, size_t n, const int64_t* target, const uint32_t* gaining) {
    if (bad_sim(e, i) || (n && (!target || !gaining))) return fail(CPM_E_ARG, "bad engine, index or buffer");
    if (n == 0) return ok();
    const SimLayout& L = e->sims.layout(i);
    for (size_t m = 0; m < n; ++m) {
        int64_t f = target[m];
        if (f < 0 || f >= L.g.n_padded) return fail(CPM_E_ARG, "target outside the lattice");
        for (int d = 0; d < L.g.D; ++d) {
            const int64_t c = f / L.g.strides[d];
            f %= L.g.strides[d];
            if (c == 0 || c == L.g.pdims[d] - 1) return fail(CPM_E_ARG, "target is a halo site");
        }
        if (gaining[m] > (uint32_t)L.n_cells) return fail(CPM_E_ARG, "gaining cell id out of range");
    }
    int64_t* d_t = nullptr;
    uint32_t* d_g = nullptr;
    cudaStream_t st = e->sims.stream();
    cudaError_t ce = cudaMalloc(&d_t, n * 8);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_g, n * 4);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_t, target, n * 8, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_g, gaining, n * 4, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cpmgpu::launch_commit_moves(L.g.D, L.NE, e->sims.device_desc(i), (int64_t)n, d_t, d_g, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    cudaFree(d_t); cudaFree(d_g);
    if (ce != cudaSuccess) return fail(CPM_E_CUDA, std::string("CUDA error: ") + cudaGetErrorString(ce));
    return ok();
}

extern "C" void cpm_engine_destroy(cpm_engine* e) { delete e; }

// ---------------------------------------------------------- many-run ----
extern "C" int cpm_run_many(const cpm_builder* const* builders, size_t n, uint64_t burn, uint64_t readout,
                            uint64_t interval, int32_t include_lattice, int32_t topology, cpm_result** out) {
    if (!builders || !out) return fail(CPM_E_ARG, "null argument");
    std::vector<Config> cfgs;
    std::vector<Initial> inits;
    const auto t0 = std::chrono::steady_clock::now();
    int rc = prepare(builders, n, cfgs, inits, burn, readout, interval);
    if (rc) return rc;
    const uint64_t place_us =
        (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
    ReadoutOptions ro;
    ro.include_lattice = include_lattice != 0;
    ro.topology = topology != 0;
    std::vector<Result> rs;
    const std::string msg = run_many(cfgs, inits, ro, rs);
    if (!msg.empty()) return fail(code_for(msg), msg);
    for (auto& r : rs)
        if (r.stats.size() > CPM_STAT_HOST_PLACE_US) r.stats[CPM_STAT_HOST_PLACE_US] = place_us;
    for (size_t i = 0; i < n; ++i) {
        auto r = std::make_unique<cpm_result>();
        r->r = std::move(rs[i]);
        out[i] = r.release();
    }
    return ok();
}

// ------------------------------------------------------ host-only helpers ----
extern "C" int cpm_builder_initial_state(const cpm_builder* b, uint32_t* lattice_out, size_t cap, uint32_t* type_of_out,
                                         size_t* n_cells, int32_t* used_default) {
    if (!b || !n_cells) return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve(b, 1, 1, 1, c);
    if (e) return e;
    std::string msg = validate(c);
    if (!msg.empty()) return fail(CPM_E_CONFIG, msg);
    Initial init;
    msg = initialize(c, init);
    if (!msg.empty()) return fail(CPM_E_INIT, msg);
    if (lattice_out) {
        if (cap < init.lattice.size()) return fail(CPM_E_ARG, "lattice buffer too small");
        std::memcpy(lattice_out, init.lattice.data(), init.lattice.size() * 4);
    }
    if (type_of_out) {
        if (*n_cells < init.type_of.size()) return fail(CPM_E_ARG, "type_of buffer too small");
        std::memcpy(type_of_out, init.type_of.data(), init.type_of.size() * 4);
    }
    *n_cells = init.type_of.size();
    if (used_default) *used_default = init.used_default;
    return ok();
}

extern "C" int cpm_builder_hashes(const cpm_builder* b, uint64_t burn, uint64_t readout, uint64_t interval,
                                  const uint32_t* lattice, size_t lattice_len, const uint32_t* type_of, size_t n_cells,
                                  char* conv_out, char* model_out) {
    if (!b || !conv_out || !model_out || (lattice_len && !lattice) || (n_cells && !type_of))
        return fail(CPM_E_ARG, "null argument");
    Config c;
    int e = resolve(b, burn, readout, interval, c);
    if (e) return e;
    const std::string ch = convention_hash(c);
    const std::string mh = model_hash(c, std::vector<uint32_t>(lattice, lattice + lattice_len),
                                      std::vector<uint32_t>(type_of, type_of + n_cells));
    std::memcpy(conv_out, ch.c_str(), 65);
    std::memcpy(model_out, mh.c_str(), 65);
    return ok();
}

extern "C" uint64_t cpm_derive_seed_u64(uint64_t master, uint64_t index) { return derive_seed_u64(master, index); }

extern "C" int cpm_tuning_report(char* buf, size_t capacity, size_t* needed) {
    const std::string r = tuning_report();
    if (needed) *needed = r.size() + 1;
    if (buf && capacity > 0) {
        const size_t n = std::min(capacity - 1, r.size());
        std::memcpy(buf, r.data(), n);
        buf[n] = 0;
    }
    return ok();
}

extern "C" int cpm_run_status(const double* energy_trace, size_t n_trace, size_t n_samples, const uint64_t* sample_mcs,
                              uint32_t n_cells, const uint32_t* volumes, const uint32_t* first_fragmented,
                              const uint32_t* last_contact_pairs, size_t n_pairs, uint32_t min_cell_volume,
                              int32_t* kind, uint32_t* cell_id, uint64_t* at_mcs) {
    if (!kind || !cell_id || !at_mcs || (n_trace && !energy_trace) || (n_samples && (!sample_mcs || !volumes)) ||
        (n_pairs && !last_contact_pairs))
        return fail(CPM_E_ARG, "null argument");
    const bool topo = first_fragmented != nullptr;
    std::vector<Sample> samples(n_samples);
    for (size_t k = 0; k < n_samples; ++k) {
        Sample& s = samples[k];
        s.mcs = sample_mcs[k];
        s.cells.resize(n_cells);
        for (uint32_t i = 0; i < n_cells; ++i) {
            s.cells[i] = CellSample();
            s.cells[i].id = i + 1;
            s.cells[i].volume = volumes[k * n_cells + i];
        }
        if (topo && first_fragmented[k]) s.fragmented.push_back(first_fragmented[k]);
        if (k + 1 == n_samples)
            for (size_t q = 0; q < n_pairs; ++q) {
                s.contact_a.push_back(last_contact_pairs[2 * q]);
                s.contact_b.push_back(last_contact_pairs[2 * q + 1]);
                s.contact_n.push_back(1);
            }
    }
    const Status st = run_status(min_cell_volume, std::vector<double>(energy_trace, energy_trace + n_trace), samples,
                                 (int)n_cells, topo);
    static const char* kinds[] = {"Ok", "NotEquilibrated", "Fragmented", "CellLost", "Degenerate"};
    *kind = 0;
    for (int q = 0; q < 5; ++q)
        if (st.kind == kinds[q]) *kind = q;
    *cell_id = st.has_cell ? st.cell_id : 0;
    *at_mcs = st.has_cell ? st.at_mcs : 0;
    return ok();
}

// ------------------------------------------------------------ serving ----
struct cpm_server {
    Server s;
};

static void copy_times(const ReqTimes& t, cpm_request_times* o) {
    if (!o) return;
    o->submitted_s = t.submitted;
    o->admitted_s = t.admitted;
    o->device_done_s = t.device_done;
    o->finished_s = t.finished;
    o->device_bytes = t.device_bytes;
}

extern "C" int cpm_serve_start(const cpm_serve_options* o, cpm_server** out) {
    if (!out) return fail(CPM_E_ARG, "null argument");
    auto sv = std::make_unique<cpm_server>();
    ServeOptions opt;
    if (o) {
        if (o->hbm_budget_bytes) opt.hbm_budget = o->hbm_budget_bytes;
        if (o->max_active > 0) opt.max_active = o->max_active;
        opt.placement_threads = o->placement_threads;
        if (o->tiled_grid_cap > 0) opt.tiled_grid_cap = o->tiled_grid_cap;
    }
    const std::string e = sv->s.start(opt);
    if (!e.empty()) return fail(CPM_E_CUDA, e);
    *out = sv.release();
    return ok();
}

extern "C" int cpm_serve_submit(cpm_server* s, const cpm_builder* b, uint64_t burn, uint64_t readout, uint64_t interval,
                                int32_t include_lattice, int32_t topology, uint64_t* ticket) {
    if (!s || !b || !ticket) return fail(CPM_E_ARG, "null argument");
    Config c;
    int rc = resolve(b, burn, readout, interval, c);
    if (rc) return rc;
    const std::string msg = validate(c);
    if (!msg.empty()) return fail(CPM_E_CONFIG, msg);
    ReadoutOptions ro;
    ro.include_lattice = include_lattice != 0;
    ro.topology = topology != 0;
    const std::string e = s->s.submit(c, ro, *ticket);
    if (!e.empty()) return fail(CPM_E_ARG, e);
    return ok();
}

static int serve_outcome(ReqState st, Result& r, const std::string& err, int32_t* state, cpm_result** out) {
    if (state) *state = (int32_t)st;
    if (st == REQ_DONE && out) {
        auto h = std::make_unique<cpm_result>();
        h->r = std::move(r);
        *out = h.release();
    }
    if (st == REQ_FAILED) return fail(code_for(err), err);
    return ok();
}

extern "C" int cpm_serve_poll(cpm_server* s, uint64_t ticket, int32_t* state, cpm_result** out,
                              cpm_request_times* times) {
    if (!s) return fail(CPM_E_ARG, "null argument");
    Result r;
    ReqTimes t;
    std::string err;
    const ReqState st = s->s.poll(ticket, out != nullptr, &r, &t, &err);
    copy_times(t, times);
    return serve_outcome(st, r, err, state, out);
}

extern "C" int cpm_serve_wait(cpm_server* s, uint64_t ticket, double timeout_s, int32_t* state, cpm_result** out,
                              cpm_request_times* times) {
    if (!s) return fail(CPM_E_ARG, "null argument");
    Result r;
    ReqTimes t;
    std::string err;
    const ReqState st = s->s.wait(ticket, timeout_s, &r, &t, &err);
    copy_times(t, times);
    return serve_outcome(st, r, err, state, out);
}

extern "C" int cpm_serve_cancel(cpm_server* s, uint64_t ticket) {
    if (!s) return fail(CPM_E_ARG, "null argument");
    if (!s->s.cancel(ticket)) return fail(CPM_E_ARG, "ticket " + std::to_string(ticket) + " is not pending");
    return ok();
}

extern "C" int cpm_serve_stats_get(cpm_server* s, cpm_serve_stats* o) {
    if (!s || !o) return fail(CPM_E_ARG, "null argument");
    const ServeStats t = s->s.stats();
    o->submitted = t.submitted;
    o->completed = t.completed;
    o->failed = t.failed;
    o->cancelled = t.cancelled;
    o->launched = t.launched;
    o->active = t.active;
    o->queued = t.queued;
    o->peak_active = t.peak_active;
    o->bytes_in_use = t.bytes_in_use;
    o->peak_bytes = t.peak_bytes;
    o->busy_seconds = t.busy_seconds;
    return ok();
}

extern "C" int cpm_serve_stop(cpm_server* s) {
    if (!s) return fail(CPM_E_ARG, "null argument");
    s->s.stop();
    delete s;
    return ok();
}

