// Host-side engine of the GB300 Cellular Potts framework (C++17).
//
// Mirrors the reference's host layers: the builder (crates/cpm-py/src/
// builder.rs:104-401), configuration resolve/validate (crates/cpm-core/src/
// config.rs:200-413), theta (theta.rs:43-178), initialisation
// (initialization.rs:39-436), the run window and readouts (output.rs:84-529),
// labelling (labelling.rs:70-154) and batch execution (batch.rs:110-153).
// The hot loop itself runs on the device (cpm_kernels.cu).
#pragma once
#include <stdint.h>

#include <array>
#include <memory>
#include <string>
#include <vector>

#include "cpm_common.h"

namespace cpmhost {

// ------------------------------------------------------------ config ----
enum Nbh { NBH_VON_NEUMANN = 0, NBH_MOORE = 1, NBH_EIGHTEEN = 2, NBH_TWENTY_SIX = 3, NBH_TWENTY_SIX_WEIGHTED = 4 };
enum Acceptance { ACC_METROPOLIS = 0, ACC_METROPOLIS_HASTINGS = 1 };
enum Proposal { PROP_UNIFORM = 0, PROP_EDGE_LIST = 1 };

struct CellType {
    std::string name;
    uint32_t target_volume = 0, target_interface = 0;
    double lambda_volume = 0, lambda_interface = 0, lambda_act = 0;
    uint32_t max_act = 0;
};
struct ActiveTerms {
    bool volume = true, interface = true, adhesion = true, act = false;
};

// ResolvedConfig (config.rs:262-282), with InitializationSpec folded in.
struct Config {
    int D = 2;
    int64_t grid[3] = {1, 1, 1};
    bool periodic = true;
    int copy_nbh = NBH_VON_NEUMANN, energy_nbh = NBH_MOORE, conn_nbh = NBH_VON_NEUMANN;
    int acceptance = ACC_METROPOLIS, proposal = PROP_UNIFORM;
    std::vector<CellType> types;
    std::vector<uint64_t> cell_counts;
    std::vector<std::vector<double>> adhesion;  // may be ragged until validated
    ActiveTerms active;
    bool init_explicit = false;
    bool warn_on_default_init = true;
    std::vector<uint32_t> init_lattice;   // unpadded row-major
    std::vector<uint64_t> init_type_of;   // per cell
    uint64_t burn_in = 0, readout = 0, interval = 0;
    uint32_t min_cell_volume = 1;
    uint64_t seed = 0;
};

int64_t n_sites(const Config& c);
// config.rs:287-413 (plus cell.rs:40-65); "" when valid.
std::string validate(const Config& c);
std::string cell_type_error(const CellType& t);
const char* nbh_name(int k);  // "VonNeumann", ...
// neighbourhood offsets in the reference order (neighborhood.rs:45-137)
std::vector<std::array<int, 3>> stencil(int kind, int D);

// theta.rs:43-178
size_t theta_len(size_t n_types);
std::vector<double> theta_extract(const Config& c);
std::vector<std::string> theta_names(const Config& c);
std::string theta_inject(Config& c, const double* theta);  // "" on success

// config.rs:479-556 — BLAKE3 over the serde_json views.
std::string convention_hash(const Config& c);
std::string model_hash(const Config& c, const std::vector<uint32_t>& lattice, const std::vector<uint32_t>& type_of);
// The same, given the configuration's convention hash.
std::string model_hash_with(const std::string& convention_hash, const std::vector<uint32_t>& lattice,
                            const std::vector<uint32_t>& type_of);
void blake3(const uint8_t* data, size_t len, uint8_t out[32]);
uint64_t derive_seed_u64(uint64_t master, uint64_t index);

// ------------------------------------------------------ initial state ----
struct Initial {
    bool used_default = false;
    std::vector<uint32_t> lattice;  // unpadded, row-major
    std::vector<uint32_t> type_of;  // per cell (index id-1)
};
// initialization.rs:39-330; "" on success.
std::string initialize(const Config& c, Initial& out);

// Padded-lattice helper (lattice.rs:24-255).
struct Geometry {
    int D;
    int64_t dims[3], pdims[3], strides[3];
    bool periodic;
    int64_t n_sites, n_padded;
    void init(const Config& c);
    int64_t flat(const int64_t* x) const;
};
std::vector<uint32_t> pad_lattice(const Geometry& g, const std::vector<uint32_t>& interior);
// (The derived per-cell state of a fresh placement, initialization.rs:396-436,
// is computed on the device: cpmgpu::launch_derive.)

// 2D simple-point table (simple_point.rs:288-306) and the FastChecker
// adjacency masks the device uses to generate the 3D table.
void simple_point_masks(int D, uint32_t* face_adj, uint32_t* full_adj, uint32_t* origin_face_mask);
void table2d(uint32_t out[8]);

// ------------------------------------------------------------ results ----
struct CellSample {
    uint32_t id, volume, interface;
    double centroid[3], eigenvalues[3], rg2, kappa2;
};
struct Sample {
    uint64_t mcs = 0;
    double energy = 0;
    std::vector<CellSample> cells;
    // contact as a sparse upper-triangular list (a < b)
    std::vector<uint32_t> contact_a, contact_b, contact_n;
    std::vector<uint32_t> fragmented;
    std::vector<uint32_t> medium_volumes;
    std::vector<uint8_t> medium_touches;
    std::vector<uint32_t> lattice;  // empty unless requested
    bool has_lattice = false;
};
struct Status {
    std::string kind = "Ok";
    bool has_cell = false;
    uint32_t cell_id = 0;
    uint64_t at_mcs = 0;
};
struct Metadata {
    std::string cpm_version, convention_hash, model_hash, seed_policy;
    uint32_t convention_version = 1, theta_layout_version = 1;
    uint64_t seed = 0;
    double derived_phi = 0;
};
struct Result {
    int D = 2;
    std::vector<int64_t> grid;
    Metadata metadata;
    Status status;
    std::vector<Sample> samples;
    std::vector<uint32_t> cell_type_index;
    std::vector<std::string> cell_type_names;
    bool used_default = false;
    std::vector<uint64_t> stats;  // CPM_STAT_* counters
    std::vector<double> energy_trace;  // burn-in energy trace (the status reads it)
};

// The run status (output.rs:456-522) from the burn-in energy trace and the
// readout samples (per-cell volumes by id, fragmented ids, the last
// sample's contact pairs); topology-based kinds only with `have_topology`.
Status run_status(uint32_t min_cell_volume, const std::vector<double>& trace, const std::vector<Sample>& samples,
                  int n_cells, bool have_topology);

// The tiled sweep's grid tuner: its table as JSON text (one object per
// lattice shape: the candidate grids with their best time per MCS in
// microseconds, and the grid chosen).
std::string tuning_report();

// Readout knobs: what each sample carries besides the per-cell summary.
struct ReadoutOptions {
    bool include_lattice = false;  // Sample.lattice
    bool topology = true;          // contact graph + labelling (needs lattice snapshots)
};

// Run many simulations (one per config) on the device in one persistent
// launch per (D, energy stencil) group; results in input order.
// `initials[i]` must be the initial state of `configs[i]`.
std::string run_many(const std::vector<Config>& configs, const std::vector<Initial>& initials,
                     const ReadoutOptions& ro, std::vector<Result>& out, int device_grid = 0);

// The drop-in `run` (builder.rs:432-474 + output.rs:434-529).
std::string run_one(const Config& c, const ReadoutOptions& ro, Result& out);
// The drop-in `run_batch` (batch.rs:110-153). On failure `stage` names the
// step that failed: BATCH_THETA (length or injection), BATCH_CONFIG
// (validation of an injected configuration), BATCH_INIT (placement) or
// BATCH_RUN (the device run).
enum BatchStage { BATCH_OK = 0, BATCH_THETA, BATCH_CONFIG, BATCH_INIT, BATCH_RUN };
std::string run_batch(const Config& base, const std::vector<std::vector<double>>& thetas, uint64_t master_seed,
                      const ReadoutOptions& ro, std::vector<Result>& out, BatchStage* stage = nullptr);

std::string last_cuda_error();
// Sets the message cpm_last_error() reports on this thread.
void set_last_error(const std::string& m);

}  // namespace cpmhost
