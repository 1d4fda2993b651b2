// cpm_run_mcs_noalloc: the MCS sweep on caller-owned device buffers, with
// no device allocation at all.
//
// Who needs it: callers that cannot (or must not) call cudaMalloc while
// they drive the simulation — a host framework that owns every device byte
// through its own pool, a service that pre-reserves all memory at start-up
// and treats any later allocation as a failure, or code running where the
// CUDA allocator is unavailable to it. They hand over the lattice and the
// per-cell arrays already resident on the device; the engine must not add
// allocations of its own behind their back.
//
// The sweep still needs a little scratch of its own (the simulation
// descriptor the kernels read, the run plan, the work-queue counter, the
// statistics counters when the caller passes none, and the per-cell conflict
// slots when the cells do not fit in shared memory). It lives in the static
// device array below, of fixed size kNoallocScratchBytes (1 MiB): every GPU
// that loads this library holds that array until the process exits.
//
// In host code `g_noalloc_scratch` is only a host-side stand-in for the
// device symbol, not a device address: a kernel given it would fault, or,
// where the GPU can reach host memory, silently use the wrong memory. The
// device address is obtained once per device, with that device current,
// through cudaGetSymbolAddress, on the first call of the entry point on that
// device; that first call should therefore come before any stream capture.
// The address is kept for the life of the process (a cudaDeviceReset of the
// device would leave it stale).
//
// Which sweep runs: the engine's resident sweep when the lattice fits one
// SM's shared memory (the same trajectory as cpm_engine_run_mcs), else the
// global-memory sweep on one CTA, which the engine only runs when forced
// (CPM_GPU_FORCE_GLOBAL); the engine's tiled sweep for such lattices needs
// per-launch scratch sized by its grid, which this entry point does not hold.
//
// Every call shares the array and the array keeps the last call's contents:
// the work-queue counter (and the fallback statistics) are cleared by each
// call, and calls that overlap on the GPU (on different streams, or from
// different threads) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/cpm_gpu.h"
#include "cpm_common.h"
#include "cpm_host.h"
#include "cpm_kernels.h"

namespace {

constexpr size_t kNoallocScratchBytes = 1u << 20;  // 1 MiB
constexpr size_t kOffDesc = 0;
constexpr size_t kOffPlan = 2048;
constexpr size_t kOffNext = 2304;
constexpr size_t kOffStats = 2560;
constexpr size_t kOffSlots = 4096;
// conflict slots: one u64 per cell id (0..n_cells)
constexpr uint64_t kNoallocMaxCells = (kNoallocScratchBytes - kOffSlots) / 8 - 1;
static_assert(sizeof(SimDesc) <= kOffPlan - kOffDesc, "descriptor does not fit its scratch region");
static_assert(sizeof(RunPlan) <= kOffNext - kOffPlan, "plan does not fit its scratch region");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_mu;
void* g_addr[64] = {nullptr};

int fail(int code, const std::string& m) {
    cpmhost::set_last_error(m);  // reported by cpm_last_error()
    return code;
}

// The 8 Moore offsets in the reference's order (neighborhood.rs:75-95:
// base-3 code, axis-0 digit fastest, origin skipped).
void moore2d(int o[8][2]) {
    int k = 0;
    for (int code = 0; code < 9; ++code) {
        if (code == 4) continue;
        o[k][0] = code % 3 - 1;
        o[k][1] = code / 3 - 1;
        ++k;
    }
}

uint32_t flood8(uint32_t comp, uint32_t universe, const uint32_t* adj) {
    for (;;) {
        uint32_t before = comp;
        for (int i = 0; i < 8; ++i)
            if ((comp >> i) & 1u) comp |= adj[i] & universe;
        if (comp == before) return comp;
    }
}

// 2D simple-point table on the stack (simple_point.rs:242-306).
void table2d_local(uint32_t out[8]) {
    int o[8][2];
    moore2d(o);
    uint32_t face[8], full[8], origin = 0;
    for (int i = 0; i < 8; ++i) {
        face[i] = full[i] = 0;
        if (std::abs(o[i][0]) + std::abs(o[i][1]) == 1) origin |= 1u << i;
        for (int j = 0; j < 8; ++j) {
            if (i == j) continue;
            const int a = std::abs(o[i][0] - o[j][0]), b = std::abs(o[i][1] - o[j][1]);
            if (a + b == 1) face[i] |= 1u << j;
            if (a <= 1 && b <= 1) full[i] |= 1u << j;
        }
    }
    for (int w = 0; w < 8; ++w) out[w] = 0;
    for (uint32_t obj = 0; obj < 256; ++obj) {
        const uint32_t cm = (~obj) & 0xFFu;
        int comps = 0;
        for (uint32_t rem = cm; rem;) { rem &= ~flood8(1u << __builtin_ctz(rem), cm, full); ++comps; }
        if (comps != 1) continue;
        int touching = 0;
        for (uint32_t rem = obj; rem;) {
            const uint32_t cc = flood8(1u << __builtin_ctz(rem), obj, face);
            rem &= ~cc;
            if (cc & origin) ++touching;
        }
        if (touching == 1) out[obj >> 5] |= 1u << (obj & 31);
    }
}

}  // namespace

extern "C" int cpm_run_mcs_noalloc(cpm_device_sim* sim, uint64_t n_mcs, void* stream) {
    using namespace cpmhost;
    if (!sim) return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: null simulation");
    if (sim->dim != 2)
        return fail(CPM_E_UNSUPPORTED,
                    "cpm_run_mcs_noalloc runs 2D lattices only (3D needs the 8 MiB simple-point table; use cpm_engine_*)");
    if (!sim->sigma || !sim->type_plus_one || !sim->volume || !sim->interface || !sim->sum_position ||
        !sim->sum_position_outer || !sim->adhesion || !sim->lambda_volume || !sim->lambda_interface ||
        !sim->target_volume || !sim->target_interface)
        return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: a device buffer pointer is null");
    if (sim->energy_neighborhood != 0 && sim->energy_neighborhood != 1)
        return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: energy_neighborhood must be 0 (von Neumann) or 1 (Moore)");
    if (sim->dims[0] < 1 || sim->dims[1] < 1)
        return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: every grid dimension must be nonzero");
    if (sim->n_types < 1) return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: at least one cell type is required");
    if ((uint64_t)sim->n_cells > kNoallocMaxCells)
        return fail(CPM_E_BUDGET, "cpm_run_mcs_noalloc: " + std::to_string(sim->n_cells) +
                                      " cells exceed the scratch limit of " + std::to_string(kNoallocMaxCells) +
                                      " cells (1 MiB static scratch); use cpm_engine_* for larger simulations");
    const int64_t padded = (sim->dims[0] + 2) * (sim->dims[1] + 2);
    if (padded >= ((int64_t)1 << 31)) return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: lattice too large");
    if (n_mcs == 0) return CPM_OK;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(CPM_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(CPM_E_ARG, "cpm_run_mcs_noalloc: device index out of range");
    char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return fail(CPM_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_addr[dev] = p;
        }
        base = (char*)g_addr[dev];
    }

    // ---- descriptor of the caller's simulation
    Config c;
    c.D = 2;
    c.grid[0] = sim->dims[0];
    c.grid[1] = sim->dims[1];
    c.periodic = sim->periodic != 0;
    Geometry g;
    g.init(c);
    SimDesc s;
    std::memset(&s, 0, sizeof s);
    s.D = 2;
    s.periodic = c.periodic;
    for (int d = 0; d < 3; ++d) {
        s.dims[d] = (int32_t)g.dims[d];
        s.pdims[d] = (int32_t)g.pdims[d];
        s.strides[d] = g.strides[d];
    }
    s.n_sites = g.n_sites;
    s.n_padded = g.n_padded;
    s.n_colors = 1;
    s.max_class = 1;
    for (int d = 0; d < 3; ++d) {
        if (d >= 2) { s.ncol[d] = 1; s.lim[d] = 1; continue; }
        const int64_t Ld = g.dims[d];
        if (Ld == 1) { s.ncol[d] = 1; s.lim[d] = 1; }
        else if (c.periodic && (Ld & 1)) { s.ncol[d] = 3; s.lim[d] = (int32_t)(Ld - 1); }
        else { s.ncol[d] = 2; s.lim[d] = (int32_t)Ld; }
        s.n_colors *= s.ncol[d];
        s.max_class *= (s.lim[d] + 1) / 2;
    }
    // copy: von Neumann [+e0, -e0, +e1, -e1] (neighborhood.rs:45-56)
    s.n_copy = 4;
    s.copy_off[0] = g.strides[0];
    s.copy_off[1] = -g.strides[0];
    s.copy_off[2] = g.strides[1];
    s.copy_off[3] = -g.strides[1];
    const int ekind = sim->energy_neighborhood == 1 ? NBH_MOORE : NBH_VON_NEUMANN;
    int mo[8][2];
    moore2d(mo);
    int ev[8][2];
    if (ekind == NBH_MOORE) {
        s.n_energy = 8;
        for (int k = 0; k < 8; ++k) { ev[k][0] = mo[k][0]; ev[k][1] = mo[k][1]; }
    } else {
        s.n_energy = 4;
        const int vn[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
        for (int k = 0; k < 4; ++k) { ev[k][0] = vn[k][0]; ev[k][1] = vn[k][1]; }
    }
    for (int k = 0; k < s.n_energy; ++k) {
        s.energy_off[k] = ev[k][0] * g.strides[0] + ev[k][1] * g.strides[1];
        s.energy_vec[k][0] = (int8_t)ev[k][0];
        s.energy_vec[k][1] = (int8_t)ev[k][1];
        s.energy_vec[k][2] = 0;
        for (int d = 0; d < 2; ++d) {
            if (ev[k][d] > 0) { s.energy_pos_mask |= 1u << k; break; }
            if (ev[k][d] < 0) break;
        }
    }
    for (int k = 0; k < 8; ++k) s.topo_off[k] = mo[k][0] * g.strides[0] + mo[k][1] * g.strides[1];
    table2d_local(s.table2d);
    s.n_types = sim->n_types;
    s.min_cell_volume = sim->min_cell_volume;
    s.seed = sim->seed;
    s.J = sim->adhesion;
    s.lambda_v = sim->lambda_volume;
    s.lambda_i = sim->lambda_interface;
    s.target_v = sim->target_volume;
    s.target_i = sim->target_interface;
    s.n_cells = (int32_t)sim->n_cells;
    s.sigma = sim->sigma;
    s.adh_of = sim->type_plus_one;
    s.volume = sim->volume;
    s.interface = sim->interface;
    s.sum_pos = sim->sum_position;
    s.sum_outer = sim->sum_position_outer;
    s.slots = (unsigned long long*)(base + kOffSlots);
    s.stats = sim->stats ? (unsigned long long*)sim->stats : (unsigned long long*)(base + kOffStats);
    s.mcs = sim->mcs;

    RunPlan p;
    std::memset(&p, 0, sizeof p);
    p.sim = 0;
    p.burn_in = n_mcs;
    p.interval = n_mcs;
    p.energy_sample_start = ~0ull;

    cudaStream_t st = (cudaStream_t)stream;
    e = cudaMemcpyAsync(base + kOffDesc, &s, sizeof s, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + kOffPlan, &p, sizeof p, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffNext, 0, 256, st);
    if (e == cudaSuccess && !sim->stats) e = cudaMemsetAsync(base + kOffStats, 0, CPM_STAT_COUNT * 8, st);
    if (e != cudaSuccess) return fail(CPM_E_CUDA, std::string("staging the descriptor: ") + cudaGetErrorString(e));

    const int NE = ekind == NBH_MOORE ? 8 : 4;
    SimDesc* d_desc = (SimDesc*)(base + kOffDesc);
    const RunPlan* d_plan = (const RunPlan*)(base + kOffPlan);
    int* d_next = (int*)(base + kOffNext);
    const bool resident = sim->n_cells < 65535 &&
                          cpmgpu::resident_smem_bytes(g.n_padded, (int)sim->n_cells) <= cpmgpu::resident_smem_limit();
    if (resident)
        e = cpmgpu::launch_resident(2, NE, cpmgpu::resident_variant(g.n_padded, (int)sim->n_cells), 0, d_desc, d_plan, 1,
                                    d_next, nullptr,
                                    cpmgpu::resident_smem_bytes(g.n_padded, (int)sim->n_cells), 1, st);
    else
        e = cpmgpu::launch_sweep(2, NE, d_desc, d_plan, 1, d_next, nullptr, (int)sim->n_cells, 1, st);
    if (e != cudaSuccess) return fail(CPM_E_CUDA, std::string("launching the sweep: ") + cudaGetErrorString(e));
    sim->mcs += n_mcs;
    return CPM_OK;
}
