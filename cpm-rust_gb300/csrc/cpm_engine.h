// Device residency for a set of simulations (internal to the library).
//
// `DeviceSims` owns one arena allocation holding, for every simulation, the
// halo-padded sigma lattice, the per-cell arrays, the parameters and the
// run-window output buffers, plus the `SimDesc` table the kernels read.
// Lattices stay resident between calls, so `run_mcs` can be called
// repeatedly (the reference's `run_mcs` seam) and sampling intervals never
// re-upload state.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "cpm_common.h"
#include "cpm_host.h"

namespace cpmhost {

struct SimLayout {
    Geometry g;
    int NE = 0;
    int n_cells = 0;
    int n_samples = 0;  // capacity of the sample buffers
    int n_energy = 0;   // capacity of the energy output
    bool lattice_samples = false;
};

// Topology readouts of one sample (output.rs:304-337): the contact graph as
// (a < b, count) in ascending order, fragmented cell ids in ascending order,
// medium components in discovery order.
struct Topo {
    std::vector<uint32_t> contact_a, contact_b, contact_n;
    std::vector<uint32_t> fragmented;
    std::vector<uint32_t> medium_volumes;
    std::vector<uint8_t> medium_touches;
};

class DeviceSims {
   public:
    DeviceSims() = default;
    ~DeviceSims();
    DeviceSims(const DeviceSims&) = delete;
    DeviceSims& operator=(const DeviceSims&) = delete;

    // Allocates and uploads every simulation. `n_samples[i]`/`n_energy[i]`
    // size the output buffers of simulation i.
    std::string create(const std::vector<Config>& configs, const std::vector<Initial>& initials,
                       const std::vector<int>& n_samples, const std::vector<int>& n_energy, bool lattice_samples,
                       cudaStream_t stream = 0);
    // Runs one plan per simulation (plans[i].sim indexes this set); one
    // persistent launch per (D, energy stencil) group.
    std::string run(const std::vector<RunPlan>& plans, int grid_override = 0);
    std::string sync();
    // Which sweep simulation i runs: shared-memory resident, tiled
    // (cooperative, all SMs on one lattice) or the global-memory sweep.
    enum Path { RESIDENT = 0, TILED = 1, GLOBAL = 2 };
    Path path(size_t i) const;
    bool resident(size_t i) const { return path(i) == RESIDENT; }
    void force_global(bool on) { force_global_ = on; }
    // Bytes this object copied host-to-device / device-to-host so far.
    uint64_t h2d_bytes() const { return h2d_bytes_; }
    uint64_t d2h_bytes() const { return d2h_bytes_; }

    size_t size() const { return layouts_.size(); }
    const SimLayout& layout(size_t i) const { return layouts_[i]; }
    const SimDesc& host_desc(size_t i) const { return descs_[i]; }
    SimDesc* device_desc(size_t i) const { return d_descs_ + i; }
    cudaStream_t stream() const { return stream_; }

    // Downloads (blocking).
    std::string read_padded(size_t i, std::vector<uint32_t>& out) const;
    std::string read_cells(size_t i, std::vector<uint32_t>& vol, std::vector<uint32_t>& itf,
                           std::vector<int64_t>& sp, std::vector<int64_t>& so) const;
    std::string read_energy(size_t i, std::vector<double>& e) const;
    std::string read_samples(size_t i, int n, std::vector<uint32_t>& vol, std::vector<uint32_t>& itf,
                             std::vector<int64_t>& sp, std::vector<int64_t>& so, std::vector<uint32_t>* lattice) const;
    std::string read_stats(size_t i, std::vector<uint64_t>& stats) const;
    std::string read_mcs(size_t i, uint64_t& mcs) const;
    // Act term state (harness use): the per-site acquisition MCS and the
    // completed-MCS counter.
    std::string write_act_state(size_t i, const std::vector<uint32_t>* birth, uint64_t mcs);
    std::string read_birth(size_t i, std::vector<uint32_t>& birth) const;
    // Topology readouts of the first ns[m] lattice snapshots of simulation
    // sims[m] (needs lattice samples), computed on the device on the
    // object's stream after the work already queued there; blocking.
    std::string topology(const std::vector<size_t>& sims, const std::vector<int>& ns,
                         std::vector<std::vector<Topo>>& out);
    // Writes sigma/V/I (harness use: set an arbitrary state).
    std::string write_state(size_t i, const std::vector<uint32_t>& padded, const std::vector<uint32_t>& vol,
                            const std::vector<uint32_t>& itf, const std::vector<int64_t>* sp = nullptr,
                            const std::vector<int64_t>* so = nullptr);
    // Replaces the descriptor of simulation i (host copy and, asynchronously
    // on the object's stream, the device copy): the serving loop points the
    // output buffers at the slice of the run window a launch produces.
    std::string set_desc(size_t i, const SimDesc& d);
    // Device bytes this object allocated (arena, descriptors, plan table).
    size_t device_bytes() const { return device_bytes_; }
    // Before create(): allocate and free in stream order on the object's
    // stream (which must then outlive the object).
    void set_stream_ordered(bool on) { stream_ordered_ = on; }
    // Caps the grid of tiled launches (the trajectory does not depend on it).
    void set_tiled_grid_cap(int cap) { tiled_grid_cap_ = cap; }
    // Before create(): host-mapped per-simulation flags the resident sweep
    // sets when a simulation's run plan ends, so its read-back can start
    // while others still run.
    void set_done_tracking(bool on) { track_done_ = on; }
    bool done(size_t i) const { return done_host_ && ((volatile uint32_t*)done_host_)[i] != 0u; }

   private:
    std::vector<SimLayout> layouts_;
    std::vector<SimDesc> descs_;
    SimDesc* d_descs_ = nullptr;
    RunPlan* d_plans_ = nullptr;
    int* d_next_ = nullptr;
    size_t plans_cap_ = 0;
    char* arena_ = nullptr;
    cudaStream_t stream_ = 0;
    bool force_global_ = false;
    bool force_tiled_ = false;
    bool no_connectivity_ = false;
    bool no_skip_ = false;        // CPM_GPU_NO_SKIP: the resident sweep builds every site
    bool prefer_tiled_ = false;
    void* d_bar_ = nullptr;
    uint32_t* d_reg_ = nullptr;  // tiled sweep: per-CTA cell registries
    size_t reg_cap_ = 0;
    std::vector<size_t> tiled_ran_;
    std::string run_tiled(const RunPlan& p, const uint64_t* t3);
    uint64_t h2d_bytes_ = 0;
    mutable std::atomic<uint64_t> d2h_bytes_{0};
    size_t device_bytes_ = 0;
    bool stream_ordered_ = false;
    int tiled_grid_cap_ = 0;
    bool track_done_ = false;
    uint32_t* done_host_ = nullptr;  // pinned, mapped
    std::vector<cudaStream_t> aux_;  // further kernel groups of one run
    std::vector<cudaEvent_t> joins_;
    cudaEvent_t ev_fork_ = nullptr;
    cudaError_t dev_alloc(void** p, size_t bytes);
    void dev_free(void* p);
};

// The whole-window plan of a configuration (output.rs:441-468) and the
// number of burn-in energy-trace points it records.
RunPlan plan_for(const Config& c, int sim, bool write_lattice);
int trace_points(uint64_t burn_in, uint64_t interval, uint64_t start);
// Reads simulation i back after its run window and builds its result. With
// ro.topology the samples' topology and the status are left to
// attach_topology.
std::string assemble_result(const Config& c, const Initial& init, const DeviceSims& dev, size_t i, int ns, int nt,
                            const ReadoutOptions& ro, Result& R);
// Moves one simulation's topology readouts into its samples and sets the
// run status (which depends on them).
void attach_topology(const Config& c, std::vector<Topo>& topo, Result& R);
// Device bytes DeviceSims::topology needs for one simulation.
size_t topology_bytes(int64_t n_sites, int n_cells);

// The 8 MiB 3D simple-point table of the current device (generated once).
const uint64_t* device_table3d(std::string& err);
int energy_count(int D, int kind);

}  // namespace cpmhost
