// Internal interface between the host engine (cpm_engine.cpp) and the
// sm_103a kernels (cpm_kernels.cu). Not part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "cpm_common.h"

namespace cpmgpu {
int sweep_block();
int sweep_max_smem_cells();
size_t sweep_smem_bytes(int max_cells);
cudaError_t launch_sweep(int D, int NE, SimDesc* d_sims, const RunPlan* d_plans, int n_plans, int* d_next,
                         const uint64_t* d_t3, int max_cells, int grid, cudaStream_t st);
cudaError_t launch_evaluate(int D, int NE, const SimDesc* d_sim, int64_t n, const int64_t* d_t, const int32_t* d_k,
                            const double* d_u, MoveOut* d_out, const uint64_t* d_t3, cudaStream_t st);
cudaError_t launch_commit_moves(int D, int NE, const SimDesc* d_sim, int64_t n, const int64_t* d_t,
                                const uint32_t* d_g, cudaStream_t st);
cudaError_t launch_recount(int D, int NE, const SimDesc* d_sim, int64_t n_sites, uint32_t* d_vol, uint32_t* d_itf,
                           cudaStream_t st);
cudaError_t launch_energy(int D, int NE, const SimDesc* d_sim, double* d_out, cudaStream_t st);
cudaError_t launch_table3d(uint64_t* d_words, const uint32_t* d_face, const uint32_t* d_full, uint32_t origin_mask,
                           cudaStream_t st);
// Shared-memory-resident sweep (cpm_resident_impl.cuh): one CTA per simulation;
// variant 1 = 256 threads (two per SM) for simulations needing at most half
// an SM's shared memory, variant 0 = 512 threads.
int resident_variant(int64_t n_padded, int n_cells);
// Raise the kernels' shared-memory limits once per device (before launches).
cudaError_t prepare_resident_kernels();
cudaError_t prepare_tiled_kernels();
size_t resident_smem_bytes(int64_t n_padded, int n_cells);
size_t resident_smem_limit();
int resident_block(int variant);
// `modes`: the simulations use Metropolis-Hastings acceptance or the Act
// term (kernels of cpm_resident_modes.cu); a launch serves one kind.
cudaError_t launch_resident(int D, int NE, int variant, int modes, SimDesc* d_sims, const RunPlan* d_plans,
                            int n_plans, int* d_next, const uint64_t* d_t3, size_t smem, int grid, cudaStream_t st);
cudaError_t resident_occupancy(int D, int NE, int variant, int modes, size_t smem, int* blocks_per_sm);
// The variants behind them.
cudaError_t prepare_resident_kernels_plain();
cudaError_t prepare_resident_kernels_modes();
cudaError_t launch_resident_plain(int D, int NE, int variant, SimDesc* d_sims, const RunPlan* d_plans, int n_plans,
                                  int* d_next, const uint64_t* d_t3, size_t smem, int grid, cudaStream_t st);
cudaError_t launch_resident_modes(int D, int NE, int variant, SimDesc* d_sims, const RunPlan* d_plans, int n_plans,
                                  int* d_next, const uint64_t* d_t3, size_t smem, int grid, cudaStream_t st);
cudaError_t resident_occupancy_plain(int D, int NE, int variant, size_t smem, int* blocks_per_sm);
cudaError_t resident_occupancy_modes(int D, int NE, int variant, size_t smem, int* blocks_per_sm);
// Tiled cooperative sweep for large lattices (cpm_tiled.cu).
bool tiled_plan(int D, const int* dims, int periodic, int* nt, int* max_box);
size_t tiled_smem_bytes(int max_box, int n_cells, int cl_cap, int D, int reg_smem);
size_t tiled_table_bytes(int n_types, int tab_n);
int tiled_block();
// `odd`: the lattice has an odd periodic side (kernels of cpm_tiled_odd.cu).
// `modes`: Metropolis-Hastings acceptance or the Act term (kernels of
// cpm_tiled_modes.cu / cpm_tiled_modes_odd.cu).
// `reg_smem`: each CTA's cell registry (stamps and box slots) in shared
// memory; else `d_registry` holds it: 2 x grid x (n_cells + 1) words.
cudaError_t tiled_occupancy(int D, int NE, int odd, int modes, size_t smem, int* per_sm);
cudaError_t launch_tiled(int D, int NE, int odd, int modes, SimDesc* d_sim, uint64_t n_mcs, const int* nt,
                         void* d_barrier, unsigned long long* d_claims, uint32_t* d_registry, const uint64_t* d_t3,
                         int max_box, int tables_in_smem, int barrier_extra, int cl_cap, int reg_smem, size_t smem,
                         int grid, cudaStream_t st, int n_cells);
// The variants behind them (even site colouring / odd periodic sides, each
// for the Metropolis chain and for the modes).
#define CPM_TILED_VARIANT_DECLS(sfx)                                                                              \
    cudaError_t prepare_tiled_kernels_##sfx();                                                                    \
    cudaError_t tiled_occupancy_##sfx(int D, int NE, size_t smem, int* per_sm);                                   \
    cudaError_t launch_tiled_##sfx(int D, int NE, SimDesc* d_sim, uint64_t n_mcs, const int* nt, void* d_barrier, \
                                   unsigned long long* d_claims, uint32_t* d_registry, const uint64_t* d_t3,      \
                                   int max_box, int tables_in_smem, int barrier_extra, int cl_cap, int reg_smem,  \
                                   size_t smem, int grid, cudaStream_t st, int n_cells);
CPM_TILED_VARIANT_DECLS(even)
CPM_TILED_VARIANT_DECLS(odd)
CPM_TILED_VARIANT_DECLS(modes_even)
CPM_TILED_VARIANT_DECLS(modes_odd)
#undef CPM_TILED_VARIANT_DECLS
// Initial state on the device (cpm_init_device.cu). check_explicit_lattice
// answers the lattice questions of explicit placement
// (initialization.rs:61-137) for a row-major interior lattice: the first
// site whose id exceeds n_cells (-1: none), the lowest cell id without a
// site and the lowest cell id not connected under von Neumann adjacency
// (0: none). Blocking; its own stream and stream-ordered scratch.
struct ExplicitCheck {
    int64_t first_bad_site;
    uint32_t zero_volume_id;
    uint32_t disconnected_id;
};
cudaError_t check_explicit_lattice(int D, const int64_t* dims, int periodic, const uint32_t* lattice, int64_t n_sites,
                                   uint32_t n_cells, ExplicitCheck* out);
// Volume, interface and position sums of every simulation of a set from its
// padded lattice (initialization.rs:396-436); the per-cell arrays are zero on
// entry. max_sites: the largest interior site count among them.
cudaError_t launch_derive(const SimDesc* d_sims, int n_sims, int64_t max_sites, cudaStream_t st);
// Copies one sample (V, I, position sums, optional lattice) of simulation d_sim.
cudaError_t launch_sample(int D, const SimDesc* d_sim, int sample, int write_lattice, int64_t n_sites, cudaStream_t st);
// Topology readouts of lattice snapshots (cpm_readout.cu). Work is cut into
// units of readout_unit() indices per item (sites, contact-pair slots and cell
// ids share the unit grid); `d_prefix` (n_items + 1) holds each item's first
// unit. Pass 0 counts contacts, 1 builds the forest inside each unit, 2 joins
// across units, 3 finds roots and counts, per unit, the entries each output
// stream will hold (d_unit_cnt: 3 per unit, zero on entry); pass 4 writes the
// streams in index order at the exclusive prefix sums d_unit_off (3 per
// unit): contact (a, b, count) triples, medium component words, fragmented
// cell ids.
int readout_unit();
cudaError_t launch_readout(int pass, const ReadoutItem* d_items, int n_items, const int64_t* d_prefix,
                           int64_t total_units, uint32_t* d_unit_cnt, const uint64_t* d_unit_off, uint32_t* d_pairs,
                           uint32_t* d_medium, uint32_t* d_frag, cudaStream_t st);
}  // namespace cpmgpu
