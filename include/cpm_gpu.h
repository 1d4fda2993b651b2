/*
 * cpm_gpu.h — C ABI of the GB300 Cellular Potts engine (libcpm_gpu.so).
 *
 * Drop-in boundary for DebajyotiS/cpm-rust. The reference crosses its only
 * FFI boundary once per call, from Python into Rust through PyO3
 * (crates/cpm-py/src/builder.rs:104-401, convert.rs:27-256); this header is
 * the same surface as plain C: a builder that accumulates the configuration
 * exactly like the PyO3 pyclass `CPM`, run / run_batch calls that execute a
 * whole trajectory per call, opaque results with accessors, and the
 * hot-path seam (`monte_carlo::run_mcs`, crates/cpm-core/src/monte_carlo.rs:
 * 327-357) for callers that drive the lattice themselves.
 *
 * Conventions: every function returns CPM_OK (0) or a CPM_E_* code; the
 * message of the last failure on the calling thread is cpm_last_error().
 * Configuration, initialisation and theta messages are the reference's own
 * texts (config.rs:287-413, initialization.rs:61-277, theta.rs:93-147,
 * batch.rs:26-45, builder.rs:35-96). The caller owns every buffer it passes;
 * the library keeps no caller pointer after a call returns. Objects are not
 * internally synchronised: use one object per thread.
 */
#ifndef CPM_GPU_H
#define CPM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPM_OK 0
#define CPM_E_CONFIG 1      /* ConfigError / CellTypeError / parse errors (-> ValueError) */
#define CPM_E_INIT 2        /* InitError (-> ValueError) */
#define CPM_E_THETA 3       /* BatchError::WrongThetaLength / ThetaError (-> ValueError) */
#define CPM_E_CUDA 4        /* a CUDA call failed; see cpm_last_error() */
#define CPM_E_TIMEOUT 5     /* a bounded device or host wait gave up */
#define CPM_E_BUDGET 6      /* serving admission: request exceeds the HBM budget */
#define CPM_E_ARG 7         /* invalid argument (null pointer, index out of range, short buffer) */
#define CPM_E_UNSUPPORTED 8 /* a request outside an entry point's domain (cpm_run_mcs_noalloc: 2D only) */

/* Message of the last failing call on this thread ("" if none). */
const char* cpm_last_error(void);
/* Library version string, e.g. "0.2.0+gb300". */
const char* cpm_version(void);

/* ------------------------------------------------------------ builder ---
 * Replaces the PyO3 pyclass `CPM` (crates/cpm-py/src/builder.rs:104-401). */
typedef struct cpm_builder cpm_builder;

/* builder.rs:117-195 (`CPM.__new__`). energy_neighborhood, acceptance and
 * proposal may be NULL (resolved defaults). active_term_keys/values may be
 * NULL with n_active_terms = 0. */
int cpm_builder_new(const uint64_t* grid, size_t grid_len, const char* boundary, uint64_t seed,
                    const char* copy_neighborhood, const char* energy_neighborhood,
                    const char* connectivity_neighborhood, const char* acceptance, const char* proposal,
                    const char* const* active_term_keys, const int32_t* active_term_values, size_t n_active_terms,
                    cpm_builder** out);
/* builder.rs:197-241 */
int cpm_builder_register_cell_type(cpm_builder* b, const char* name, uint32_t target_volume,
                                   uint32_t target_interface, double lambda_volume, double lambda_interface,
                                   double lambda_act, uint32_t max_act);
/* builder.rs:243-254 */
int cpm_builder_add_cells(cpm_builder* b, const char* cell_type, uint64_t n);
/* builder.rs:256-262: row-major values of n_rows rows with the given lengths
 * (ragged rows are accepted here and rejected by validation at run time). */
int cpm_builder_set_adhesion(cpm_builder* b, const double* values, const size_t* row_lengths, size_t n_rows);
/* builder.rs:270-296: lattice == NULL selects the default scatter-and-grow. */
int cpm_builder_initialize(cpm_builder* b, const uint32_t* lattice, size_t lattice_len,
                           const uint64_t* cell_type_of, size_t cell_type_of_len, int32_t has_cell_type_of,
                           int32_t warn_on_default_init);
typedef struct cpm_result cpm_result;
/* builder.rs:304-333 + 432-474: resolve, validate, place, burn in, read out.
 * *used_default reports whether scatter-and-grow placement was used. */
int cpm_builder_run(const cpm_builder* b, uint64_t burn_in_mcs, uint64_t readout_mcs, uint64_t sampling_interval_mcs,
                    int32_t include_lattice, int32_t* used_default, cpm_result** out);
/* builder.rs:342-381 + 485-525 and batch.rs:110-153: thetas are
 * concatenated, theta i has theta_lengths[i] entries; per-simulation seeds
 * are derive_seed_u64(master_seed, i). out must hold n_thetas pointers. All
 * simulations run in one persistent device launch. */
int cpm_builder_run_batch(const cpm_builder* b, const double* thetas, const size_t* theta_lengths, size_t n_thetas,
                          uint64_t burn_in_mcs, uint64_t readout_mcs, uint64_t sampling_interval_mcs,
                          uint64_t master_seed, int32_t include_lattice, int32_t* any_used_default, cpm_result** out);
/* builder.rs:386-430 (theta.rs:43-178) */
int cpm_builder_theta_len(const cpm_builder* b, size_t* out);
int cpm_builder_extract_theta(const cpm_builder* b, double* out, size_t capacity);
int cpm_builder_theta_name(const cpm_builder* b, size_t index, char* buf, size_t capacity);
void cpm_builder_free(cpm_builder* b);

/* ------------------------------------------------------------ results ---
 * Replaces PyRunResult / PySample / PyRunMetadata / PyStatus
 * (crates/cpm-py/src/convert.rs:27-256). */
typedef struct {
    int32_t dim;
    int32_t n_types;
    int64_t grid[3];
    uint64_t n_cells;
    uint64_t n_samples;
    int32_t used_default;
    int32_t pad;
} cpm_result_info;

typedef struct {
    char cpm_version[32];
    char convention_hash[65];
    char model_hash[65];
    char seed_policy[32];
    uint32_t convention_version;
    uint32_t theta_layout_version;
    uint64_t seed;
    double derived_phi;
} cpm_metadata;

typedef struct {
    char kind[24]; /* "Ok", "CellLost", "Fragmented", "NotEquilibrated", "Degenerate" */
    int32_t has_cell;
    uint32_t cell_id;
    uint64_t at_mcs;
} cpm_status;

typedef struct {
    uint64_t n_contact;   /* nonzero contact pairs (a < b) */
    uint64_t n_fragmented;
    uint64_t n_medium;    /* medium components */
    int32_t has_lattice;
    int32_t pad;
} cpm_sample_sizes;

/* Caller-owned destination buffers for one sample; any pointer may be NULL
 * to skip that field. Per-cell arrays have n_cells rows in id order. */
typedef struct {
    uint64_t* mcs;
    double* conservative_energy;
    uint32_t* ids;
    uint32_t* volume;
    uint32_t* interface;
    double* centroid;      /* n_cells x dim */
    double* eigenvalues;   /* n_cells x dim, descending */
    double* radius_of_gyration_sq;
    double* kappa_sq;
    uint32_t* contact_a;   /* n_contact; canonical (min, max) pairs, medium = 0 */
    uint32_t* contact_b;
    uint32_t* contact_count;
    uint32_t* fragmented_cells;
    uint32_t* medium_component_volumes;
    uint8_t* medium_component_touches_boundary;
    uint32_t* lattice;     /* product(grid), row-major; only if has_lattice */
} cpm_sample_out;

int cpm_result_info_get(const cpm_result* r, cpm_result_info* out);
int cpm_result_metadata_get(const cpm_result* r, cpm_metadata* out);
int cpm_result_status_get(const cpm_result* r, cpm_status* out);
int cpm_result_cell_type_index(const cpm_result* r, uint32_t* out /* n_cells */);
int cpm_result_cell_type_name(const cpm_result* r, size_t type_index, char* buf, size_t capacity);
int cpm_result_sample_sizes(const cpm_result* r, size_t sample, cpm_sample_sizes* out);
int cpm_result_sample_read(const cpm_result* r, size_t sample, const cpm_sample_out* out);

/* All samples of a result in one call (the same fields as
 * cpm_result_sample_read, samples back to back): the fixed-size fields as
 * n_samples x n_cells (x D) arrays, the variable-size ones concatenated with
 * n_samples + 1 offsets, lattices as n_samples x N_sites when present. No
 * reference counterpart (a bulk form of the per-sample accessors). */
typedef struct {
    uint64_t n_samples, n_cells;
    uint64_t total_contact, total_fragmented, total_medium;
    int32_t has_lattice;
    int32_t pad;
} cpm_samples_sizes;
int cpm_result_samples_sizes(const cpm_result* r, cpm_samples_sizes* out);

typedef struct {
    uint64_t* mcs;
    double* conservative_energy;
    uint32_t *ids, *volume, *interface;
    double *centroid, *eigenvalues, *radius_of_gyration_sq, *kappa_sq;
    uint64_t* contact_offsets;
    uint32_t *contact_a, *contact_b, *contact_count;
    uint64_t* fragmented_offsets;
    uint32_t* fragmented_cells;
    uint64_t* medium_offsets;
    uint32_t* medium_component_volumes;
    uint8_t* medium_component_touches_boundary;
    uint32_t* lattice;
} cpm_samples_out;
int cpm_result_samples_read(const cpm_result* r, const cpm_samples_out* out);
/* cpm_result_samples_read for n results at once (results[i] into outs[i]),
 * spread over the host's cores: the read-back of a whole batch. */
int cpm_results_samples_read(const cpm_result* const* results, size_t n, const cpm_samples_out* outs);
/* Device counters of the run (order: attempts, non-null, topology
 * rejections, guard rejections, evaluated, accepted, conflict rounds, colour
 * passes, timeouts, fixpoint iterations, h2d bytes, d2h bytes, deferred
 * moves, then cycle counters of the tiled sweep); out holds 32 values. */
int cpm_result_stats(const cpm_result* r, uint64_t* out32);
void cpm_result_free(cpm_result* r);

/* --------------------------------------------------- hot-path engine ---
 * The seam the kernels replace: monte_carlo::run_mcs (monte_carlo.rs:
 * 327-357) on device-resident lattices. An engine holds one or more
 * simulations, each built and placed from a builder (its grid, types,
 * adhesion, seed and initialisation); `run_mcs` advances every simulation
 * by n MCS in one persistent launch. Per-cell arrays are indexed by cell id
 * (n_cells + 1 entries, entry 0 = medium). */
typedef struct cpm_engine cpm_engine;

typedef struct {
    int32_t dim;
    int32_t periodic;
    int64_t dims[3];
    int64_t padded_dims[3];
    int64_t strides[3];
    uint64_t n_sites;
    uint64_t n_padded;
    uint64_t n_cells;
    int32_t n_energy;   /* energy-neighbourhood size */
    int32_t n_colors;   /* checkerboard colours per MCS */
} cpm_sim_info;

/* Per-move parity record (monte_carlo.rs:52-145 decided with explicit
 * draws): k indexes the von Neumann copy stencil, u is the uniform draw used
 * when delta_h > 0. `accepted` applies the reference's rule to the FP64
 * delta_h; `accepted_sweep` is the decision the sweeps take for the same u
 * (float pre-decision with an error bound, FP64 fallback) and must equal it. */
typedef struct {
    int64_t target_flat, source_flat;
    uint32_t losing, gaining;
    int32_t null_move, topology_ok, volume_guard_ok, evaluated;
    int32_t delta_i_losing, delta_i_gaining;
    double delta_h;
    int32_t accepted;
    int32_t accepted_sweep;
} cpm_move;

/* stream: a cudaStream_t to launch on, or NULL for the default stream. */
int cpm_engine_create(const cpm_builder* const* builders, size_t n, void* stream, cpm_engine** out);
int cpm_engine_size(const cpm_engine* e, size_t* out);
int cpm_engine_sim_info(const cpm_engine* e, size_t sim, cpm_sim_info* out);
/* Advance every simulation by n_mcs MCS (asynchronous on the engine stream). */
int cpm_engine_run_mcs(cpm_engine* e, uint64_t n_mcs);
int cpm_engine_synchronize(cpm_engine* e);
int cpm_engine_mcs(const cpm_engine* e, size_t sim, uint64_t* out);
int cpm_engine_read_lattice(const cpm_engine* e, size_t sim, uint32_t* out /* n_sites */);
int cpm_engine_read_padded(const cpm_engine* e, size_t sim, uint32_t* out /* n_padded */);
int cpm_engine_read_cells(const cpm_engine* e, size_t sim, uint32_t* volume, uint32_t* interface, int64_t* sum_position,
                          int64_t* sum_position_outer);
/* Global energy of the current state (energy.rs:104-308), computed on the device. */
int cpm_engine_energy(const cpm_engine* e, size_t sim, double* out);
/* Full recount of volume and interface from the lattice on the device
 * (checker.rs:36-83); *ok = 1 iff it equals the incrementally kept state. */
int cpm_engine_recount_check(const cpm_engine* e, size_t sim, int32_t* ok, uint32_t* volume, uint32_t* interface);
int cpm_engine_stats(const cpm_engine* e, size_t sim, uint64_t* out32);
/* One sample of the current state (output.rs:304-337 `take_sample`, the
 * `cpm_sample` seam): per-cell volume, interface, centroid and gyration,
 * the contact graph and the labelling, all computed on the device, returned
 * as a result with one sample (its energy is the device's global energy of
 * the state, its mcs the MCS completed so far). Free with cpm_result_free. */
int cpm_engine_take_sample(cpm_engine* e, size_t sim, int32_t include_lattice, cpm_result** out);
/* Parity harness for the Act term (energy.rs:329-471): set the per-site
 * acquisition MCS (n_padded values, padded indexing as `birth_mcs`; null
 * keeps it) and the completed-MCS counter the activities are measured
 * against; read the acquisition MCS back. */
int cpm_engine_write_act_state(cpm_engine* e, size_t sim, const uint32_t* birth_padded, uint64_t mcs);
int cpm_engine_read_birth(const cpm_engine* e, size_t sim, uint32_t* out /* n_padded */);
/* Parity harness: overwrite the dynamic state, decide moves without
 * committing them, or apply moves in order with the sweep's commit. Every
 * padded entry written must be a cell id <= n_cells (CPM_E_ARG otherwise);
 * targets must be interior sites and copy directions < 2 * dim. */
int cpm_engine_write_state(cpm_engine* e, size_t sim, const uint32_t* padded, const uint32_t* volume,
                           const uint32_t* interface, const int64_t* sum_position, const int64_t* sum_position_outer);
int cpm_engine_evaluate_moves(cpm_engine* e, size_t sim, size_t n, const int64_t* target_flat, const int32_t* k,
                              const double* u, cpm_move* out);
int cpm_engine_commit_moves(cpm_engine* e, size_t sim, size_t n, const int64_t* target_flat, const uint32_t* gaining);
void cpm_engine_destroy(cpm_engine* e);

/* ------------------------------------------------------ many-run batch ---
 * Extension of run_batch for simulations that differ in grid as well as
 * theta (no counterpart in the reference, whose run_batch shares one grid):
 * one builder per simulation, all run in one persistent launch. topology=0
 * skips the contact graph and labelling (samples then carry volume,
 * interface, centroid and gyration only). */
int cpm_run_many(const cpm_builder* const* builders, size_t n, uint64_t burn_in_mcs, uint64_t readout_mcs,
                 uint64_t sampling_interval_mcs, int32_t include_lattice, int32_t topology, cpm_result** out);

/* ---------------------------------------------------- host-only helpers ---
 * No device work: the placement, hashes and seeds the reference computes on
 * the host, exposed so callers (and the CPU test suite) can check them. */
/* Resolves, validates and places (initialization.rs:39-330) without running.
 * lattice_out holds product(grid) ids, type_of_out n_cells type indices
 * (capacity in *n_cells on input, count on output). */
int cpm_builder_initial_state(const cpm_builder* b, uint32_t* lattice_out, size_t lattice_capacity,
                              uint32_t* type_of_out, size_t* n_cells, int32_t* used_default);
/* convention_hash and model_hash (config.rs:479-556) of the configuration
 * resolved with the given windows and the given lattice (product(grid) ids)
 * and cell types; each out buffer holds 65 bytes. */
int cpm_builder_hashes(const cpm_builder* b, uint64_t burn_in_mcs, uint64_t readout_mcs, uint64_t sampling_interval_mcs,
                       const uint32_t* lattice, size_t lattice_len, const uint32_t* type_of, size_t n_cells,
                       char* convention_hash_out, char* model_hash_out);
/* rng.rs:37-40: first 8 LE bytes of BLAKE3(master LE || index LE). */
uint64_t cpm_derive_seed_u64(uint64_t master_seed, uint64_t simulation_index);
/* No counterpart in the reference (it has no launch parameters). The tiled
 * sweep's grid tuner: for every lattice shape it has met in this process,
 * the grids it timed (tiles per CTA 1..4; the trajectory does not depend on
 * the grid), their best time per MCS in microseconds and the grid in use, as
 * JSON text. *needed receives the length plus one; the text is cut to fit
 * `capacity`. */
int cpm_tuning_report(char* buf, size_t capacity, size_t* needed);
/* The run status of output.rs:456-522 (SimulationStatus, with the priority
 * NotEquilibrated > Fragmented > CellLost > Degenerate) over given readouts:
 * the burn-in energy trace (not_equilibrated, output.rs:388-420), then per
 * readout sample its MCS and every cell's volume (row k holds ids 1..n_cells),
 * the first fragmented cell id of each sample (0: none; NULL: the run had no
 * topology readouts, which skips Fragmented and Degenerate) and the last
 * sample's contact pairs with a positive count (a, b interleaved; the medium
 * is id 0). kind: 0 Ok, 1 NotEquilibrated, 2 Fragmented, 3 CellLost,
 * 4 Degenerate; cell_id and at_mcs are set for Fragmented and CellLost, else 0.
 * This is the rule cpm_builder_run applies to its own samples. */
int cpm_run_status(const double* energy_trace, size_t n_trace, size_t n_samples, const uint64_t* sample_mcs,
                   uint32_t n_cells, const uint32_t* volumes, const uint32_t* first_fragmented,
                   const uint32_t* last_contact_pairs, size_t n_pairs, uint32_t min_cell_volume, int32_t* kind,
                   uint32_t* cell_id, uint64_t* at_mcs);

/* -------------------------------------------- allocation-free sweep ---
 * No counterpart in the reference. For callers that cannot call cudaMalloc
 * while they run — a host framework that owns all device memory through its
 * own pool, or a service that reserves every byte at start-up and treats a
 * later allocation as a failure — and that therefore hand over simulations
 * already resident on the device. cpm_run_mcs_noalloc advances such a
 * simulation by n_mcs MCS and allocates no device memory: its own scratch
 * (descriptor, plan, work-queue counter, per-cell conflict slots) is a
 * static 1 MiB device array inside the library, held by every GPU that
 * loads it until the process exits.
 * Which sweep runs: a lattice that fits one SM's shared memory (the
 * engine's resident sweep, about 298^2 and below) runs exactly the sweep
 * cpm_engine_run_mcs runs for it, so both give the same trajectory. A
 * larger lattice runs the global-memory sweep on one CTA (the chain the
 * engine runs under CPM_GPU_FORCE_GLOBAL), not the engine's tiled sweep:
 * a different, equally exact chain, and much slower than the engine there.
 * Limits: 2D lattices only (3D needs the 8 MiB simple-point table), at most
 * 130,559 cells. The first call on a device does the set-up: it looks up
 * the array's device address (cudaGetSymbolAddress) with that device
 * current, so make that first call before any stream capture. The address
 * is kept for the life of the process, so the library must not outlive a
 * cudaDeviceReset of that device. Calls share the array: calls that overlap
 * on the GPU race, so serialise them. On return sim->mcs has advanced by
 * n_mcs (the RNG counter base of the next call). */
typedef struct {
    int32_t dim;                  /* must be 2 */
    int32_t periodic;             /* 1 periodic, 0 fixed */
    int64_t dims[3];              /* interior extent; dims[2] ignored */
    int32_t energy_neighborhood;  /* 0 von Neumann, 1 Moore */
    int32_t n_types;
    uint32_t n_cells;
    uint32_t min_cell_volume;     /* 1 in the reference */
    uint64_t seed;
    uint64_t mcs;                 /* MCS already performed */
    /* device pointers, caller-owned; per-cell arrays are indexed by id (n_cells + 1) */
    uint32_t* sigma;              /* halo-padded lattice ((dims+2) per axis), halo consistent,
                                     every entry a cell id <= n_cells (not checked: device memory) */
    const uint16_t* type_plus_one;/* cell type + 1 per id, entry 0 = 0 (medium) */
    uint32_t* volume;
    uint32_t* interface;
    int64_t* sum_position;        /* (n_cells + 1) x 2 */
    int64_t* sum_position_outer;  /* (n_cells + 1) x 2 x 2 */
    const double* adhesion;       /* (n_types + 1)^2, row-major, 0 = medium */
    const double* lambda_volume;  /* n_types */
    const double* lambda_interface;
    const uint32_t* target_volume;
    const uint32_t* target_interface;
    uint64_t* stats;              /* optional: 32 device counters (the cpm_engine_stats layout) accumulated by the sweep */
} cpm_device_sim;

int cpm_run_mcs_noalloc(cpm_device_sim* sim, uint64_t n_mcs, void* stream);

/* ------------------------------------------------------------ serving ---
 * A device-resident request loop (no counterpart in the reference, whose
 * unit of work is one blocking `run` or `run_batch` call): simulations are
 * submitted at any time, admitted in submission order while the active ones
 * fit `max_active` slots and the HBM budget, run side by side on the device
 * (each on its own stream with its whole run window enqueued; lattices stay
 * on the device from upload to read-back), and read out and freed when
 * their windows end, which admits the next. Each result equals what
 * `cpm_builder_run` returns for the same builder and window, alone or in
 * any mix. All functions are thread-safe. */
typedef struct cpm_server cpm_server;

typedef struct {
    uint64_t hbm_budget_bytes;  /* device bytes admitted simulations may hold; 0 = 150 GiB */
    int32_t max_active;         /* simulations on the device at once; 0 = 128 */
    int32_t placement_threads;  /* host threads for placements and read-backs; 0 = automatic */
    int32_t tiled_grid_cap;     /* CTAs of one simulation on the tiled sweep; 0 = 64 */
    int32_t pad;
} cpm_serve_options;

#define CPM_REQ_PLACING 0
#define CPM_REQ_QUEUED 1
#define CPM_REQ_RUNNING 2
#define CPM_REQ_DONE 3
#define CPM_REQ_FAILED 4
#define CPM_REQ_CANCELLED 5

typedef struct {
    double submitted_s, admitted_s, device_done_s, finished_s; /* seconds since the server started */
    uint64_t device_bytes;                                     /* device bytes it held */
} cpm_request_times;

typedef struct {
    uint64_t submitted, completed, failed, cancelled, launched;
    uint64_t active, queued, peak_active;
    uint64_t bytes_in_use, peak_bytes;
    double busy_seconds;                        /* wall time with simulations on the device */
} cpm_serve_stats;

int cpm_serve_start(const cpm_serve_options* options, cpm_server** out);
/* Validates the builder's configuration with the window (as cpm_builder_run
 * does) and enqueues it; the ticket names the request from then on. */
int cpm_serve_submit(cpm_server* s, const cpm_builder* b, uint64_t burn_in_mcs, uint64_t readout_mcs,
                     uint64_t sampling_interval_mcs, int32_t include_lattice, int32_t topology, uint64_t* ticket);
/* Non-blocking. state receives CPM_REQ_*; when it is CPM_REQ_DONE and out is
 * not NULL, *out receives the result (free with cpm_result_free) and the
 * ticket is retired. A failed request returns its error code and message. */
int cpm_serve_poll(cpm_server* s, uint64_t ticket, int32_t* state, cpm_result** out, cpm_request_times* times);
/* Blocks until the request finishes or timeout_s passes (negative: no
 * limit); then as cpm_serve_poll with out. */
int cpm_serve_wait(cpm_server* s, uint64_t ticket, double timeout_s, int32_t* state, cpm_result** out,
                   cpm_request_times* times);
int cpm_serve_cancel(cpm_server* s, uint64_t ticket);
int cpm_serve_stats_get(cpm_server* s, cpm_serve_stats* out);
/* Cancels unfinished requests, stops the loop and frees the server. */
int cpm_serve_stop(cpm_server* s);

#ifdef __cplusplus
}
#endif
#endif /* CPM_GPU_H */
