// Plain-old-data layout shared by the host engine and the sm_103a kernels.
//
// One `SimDesc` describes one device-resident simulation: its halo-padded
// sigma lattice (the reference's layout, crates/cpm-core/src/lattice.rs:70-255),
// the per-cell arrays (crates/cpm-core/src/state.rs:168-248), the offset
// tables (crates/cpm-core/src/model.rs:44-76) and the parameters the local
// Delta-H needs (crates/cpm-core/src/energy.rs:72-309). Per-cell arrays are
// indexed by cell id (length n_cells + 1, slot 0 = medium, never read for
// volume/interface terms) so the hot loop needs no `id - 1` branch.
#pragma once
#include <stdint.h>

#define CPM_MAX_D 3
#define CPM_MAX_STENCIL 26

// Statistics counters per simulation (device, u64 each).
enum CpmStat {
    CPM_STAT_ATTEMPTS = 0,   // sites visited (one per site per MCS)
    CPM_STAT_NONNULL = 1,    // passed the early-out (sigma[t] != sigma[s])
    CPM_STAT_TOPO_REJECT = 2,
    CPM_STAT_GUARD_REJECT = 3,
    CPM_STAT_EVALUATED = 4,  // reached Delta-H
    CPM_STAT_ACCEPTED = 5,
    CPM_STAT_ROUNDS = 6,     // conflict-resolution rounds (summed over passes)
    CPM_STAT_PASSES = 7,         // colour passes (tiled sweep: tile passes, one per tile and site colour)
    CPM_STAT_SPIN_TIMEOUTS = 8,  // bounded waits that gave up (must stay 0)
    CPM_STAT_FIXPOINT_ITERS = 9, // fixpoint iterations summed over threads
    CPM_STAT_H2D_BYTES = 10,     // host-to-device bytes of the call (host-side count)
    CPM_STAT_D2H_BYTES = 11,     // device-to-host bytes of the call (host-side count)
    CPM_STAT_DEFERRED = 12,      // tiled sweep: moves skipped because a cell was owned by another tile
    CPM_STAT_CYC_PASSES = 13,    // tiled sweep: SM cycles in the site-colour passes (thread 0 of each CTA)
    CPM_STAT_CYC_STAGE = 14,     // tiled sweep: SM cycles staging boxes and writing them back
    CPM_STAT_CYC_SYNC = 15,      // tiled sweep: SM cycles in claims and grid barriers
    CPM_STAT_CYC_BUILD = 16,     // tiled sweep: cycles building candidate lists
    CPM_STAT_CYC_EVAL = 17,      // tiled sweep: cycles in speculative evaluation
    CPM_STAT_CYC_FIX = 18,       // tiled sweep: cycles in the fixpoint iterations
    CPM_STAT_CYC_APPLY = 19,     // tiled sweep: cycles applying and re-evaluating
    CPM_STAT_WIDE_PASSES = 20,   // tiled sweep: tile passes with more than 64 candidates (block-wide resolve)
    CPM_STAT_CYC_LOWER = 21,     // tiled sweep: cycles finding the lower-priority sharers (warp resolve)
    CPM_STAT_CYC_CLAIM = 22,     // tiled sweep: cycles registering cell claims
    CPM_STAT_CYC_BAR_CLAIM = 23, // tiled sweep: cycles waiting in the grid barrier after the claims
    CPM_STAT_CYC_BAR_WRITE = 24, // tiled sweep: cycles waiting in the grid barrier after the write-back
    CPM_STAT_EXACT_DECISIONS = 25, // decisions the float bracket left to the FP64 computation
    CPM_STAT_HOST_PREP_US = 26,  // run/run_batch/run_many: microseconds of upload and launch
    CPM_STAT_DEVICE_US = 27,     // microseconds from the launch to the end of the device work
    CPM_STAT_HOST_READ_US = 28,  // microseconds of read-back and host readouts after the device work (they overlap it)
    CPM_STAT_CYC_RES_BUILD = 29,   // resident sweep: cycles building candidate lists (thread 0)
    CPM_STAT_CYC_RES_RESOLVE = 30, // resident sweep: cycles resolving them (thread 0)
    CPM_STAT_HOST_PLACE_US = 31,   // run/run_many: microseconds of validation and initial placement
    CPM_STAT_COUNT = 32
};

struct SimDesc {
    // ---- geometry ----
    int32_t D;
    int32_t periodic;
    int32_t dims[3];
    int32_t pdims[3];
    int64_t strides[3];
    int64_t n_sites;
    int64_t n_padded;
    // checkerboard colouring: per axis 1, 2 or 3 colours; `lim` is the
    // exclusive upper coordinate of the parity colours on that axis.
    int32_t ncol[3];
    int32_t lim[3];
    int32_t n_colors;
    int32_t max_class;  // largest colour-class size
    // ---- stencils (flat padded-index deltas) ----
    int32_t n_copy;
    int32_t n_energy;
    int64_t copy_off[6];
    int64_t energy_off[CPM_MAX_STENCIL];
    int64_t topo_off[CPM_MAX_STENCIL];
    int8_t energy_vec[CPM_MAX_STENCIL][3];  // integer offset of each energy neighbour
    int8_t copy_vec[6][3];                  // integer offset of each copy neighbour
    int8_t topo_vec[CPM_MAX_STENCIL][3];    // integer offset of each simple-point neighbour
    uint32_t energy_pos_mask;               // offsets whose first nonzero component is > 0
    uint32_t table2d[8];                    // 2D simple-point table (256 bits)
    // ---- parameters ----
    int32_t n_types;
    uint32_t min_cell_volume;
    uint64_t seed;
    const double* J;                // (n_types+1)^2 row-major, 0 = medium
    const double* lambda_v;         // per type
    const double* lambda_i;
    const uint32_t* target_v;
    const uint32_t* target_i;
    // Exact FP64 tables built on the host with the reference's operations:
    // vterm[t*tab_n + x] = lambda_V[t] * ((x - V*[t])^2),
    // iterm[t*tab_n + x] = lambda_I[t] * ((x - I*[t])^2) for 0 <= x < tab_n,
    // dj[(l*(n+1) + g)*(n+1) + k] = J[g][k] - J[l][k] (adhesion difference).
    const double* vterm;
    const double* iterm;
    const double* dj;
    // The same tables and J rounded to float (round to nearest), for the
    // bounded FP32 pre-decision; null disables it. vterm32lo / iterm32lo
    // hold the remainders fl32(x - fl32(x)), so that hi + lo carries x to
    // about 2^-48 relative.
    const float* vterm32;
    const float* iterm32;
    const float* vterm32lo;
    const float* iterm32lo;
    const float* dj32;
    const float* J32;
    int32_t tab_n;
    // Test switch (the reference's `attempt(cpm, false)` of its exact-Boltzmann
    // harness): nonzero skips the connectivity check; honoured by the
    // global-memory sweep only, and the engine routes such simulations there.
    int32_t no_connectivity;
    // ---- state ----
    int32_t n_cells;
    // bit 0: the resident sweep builds every site of a chunk (no
    // active-block skip; same result); a test switch (CPM_GPU_NO_SKIP)
    int32_t sweep_flags;
    uint32_t* sigma;                // n_padded
    const uint16_t* adh_of;         // per id: type + 1 (0 for medium)
    uint32_t* volume;               // per id
    uint32_t* interface;            // per id
    int64_t* sum_pos;               // per id * D
    int64_t* sum_outer;             // per id * D * D
    unsigned long long* slots;      // per id (only when they do not fit in shared memory)
    unsigned long long* stats;      // CPM_STAT_COUNT
    uint64_t mcs;                   // MCS already completed (RNG counter base)
    // ---- run-window outputs (device) ----
    double* energy_out;             // energies written by the run plan
    uint32_t* sample_volume;        // n_samples * (n_cells+1)
    uint32_t* sample_interface;
    int64_t* sample_sum_pos;        // n_samples * (n_cells+1) * D
    int64_t* sample_sum_outer;      // n_samples * (n_cells+1) * D * D
    uint32_t* sample_lattice;       // n_samples * n_sites (unpadded) or null
    int32_t* error;                 // first error code (0 = none)
    uint32_t* done_flag;            // optional (host-mapped): set to 1 when a run plan of this simulation ends
    // ---- modes of the loop (every sweep runs them) ----
    int32_t acceptance;             // 0 = Metropolis, 1 = MetropolisHastings (monte_carlo.rs:147-196)
    int32_t act;                    // Act term active (energy.rs:329-471)
    const double* lambda_act;       // per type
    const uint32_t* max_act;        // per type
    uint32_t* birth;                // per padded site: MCS at which its current owner acquired it
};

// One unit of device work: a whole run plan for one simulation, replaying
// output.rs:434-468 (burn-in in interval-sized chunks with the energy trace
// over its final quarter, then `n_samples` readout chunks with one sample
// after each).
struct RunPlan {
    int32_t sim;
    int32_t n_samples;
    uint64_t burn_in;
    uint64_t interval;
    uint64_t energy_sample_start;  // burned_in >= this -> record energy
    uint64_t readout_chunks;       // == n_samples
    int32_t write_samples;
    int32_t write_lattice;
};

// One lattice snapshot for the device topology readouts (cpm_readout.cu):
// the snapshot and the scratch the readouts of its simulation reuse from
// sample to sample. `tri` and `ncomp` are zero on entry and left zero.
struct ReadoutItem {
    const uint32_t* lat;  // n_sites, interior, last axis fastest
    uint32_t* parent;     // n_sites: union-find forest
    uint32_t* aux;        // n_sites: medium component volume at its root, bit 31 = touches a fixed boundary
    uint32_t* tri;        // n_cells * (n_cells + 1) / 2: contact counts of the pairs a < b, row-major
    uint32_t* ncomp;      // n_cells + 1: von Neumann components per cell id
    int64_t n_sites;
    int64_t tri_n;
    int32_t dims[3];
    int32_t D;
    int32_t periodic;
    int32_t n_cells;
    int32_t energy_maxnz;  // energy stencil = offsets in {-1,0,1}^D with 1..energy_maxnz nonzero components
    int32_t pad;
};

// Per-move record of the parity harness (same layout as the oracle's).
struct MoveOut {
    int64_t target_flat, source_flat;
    uint32_t losing, gaining;
    int32_t null_move, topology_ok, volume_guard_ok, evaluated;
    int32_t delta_i_losing, delta_i_gaining;
    double delta_h;
    int32_t accepted;
    int32_t accepted_sweep;  // the sweeps' bounded decision (decide_move) on the same u
};
