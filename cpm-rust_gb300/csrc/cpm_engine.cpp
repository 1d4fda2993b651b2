// Device residency, the run window and result assembly (host side).
//
// run_many() is the GB300 form of the reference's run path: it uploads every
// simulation once, runs each one's whole run plan (burn-in + readout,
// output.rs:434-468) inside one persistent sweep launch, and then assembles
// the reference's readouts on the host from the device samples: per-cell
// volume/interface/centroid/gyration (output.rs:147-302), the contact graph
// (state.rs:127-157), labelling (labelling.rs:70-154), the run status
// (output.rs:388-522) and the metadata hashes (config.rs:479-556).
#include "cpm_engine.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>

#include "cpm_kernels.h"

namespace cpmhost {

static thread_local std::string g_cuda_error;
std::string last_cuda_error() { return g_cuda_error; }

#define CUDA_TRY(expr)                                                                   \
    do {                                                                                 \
        cudaError_t _e = (expr);                                                         \
        if (_e != cudaSuccess) {                                                         \
            g_cuda_error = std::string(#expr) + ": " + cudaGetErrorString(_e);           \
            return std::string("CUDA error: ") + cudaGetErrorString(_e) + " (" #expr ")"; \
        }                                                                                \
    } while (0)

int energy_count(int D, int kind) {
    if (kind == NBH_VON_NEUMANN) return 2 * D;
    if (kind == NBH_MOORE) return 8;
    if (kind == NBH_EIGHTEEN) return 18;
    return 26;
}

// ------------------------------------------------------------ 3D table ----
const uint64_t* device_table3d(std::string& err) {
    static std::mutex mu;
    static std::map<int, uint64_t*> tables;
    std::lock_guard<std::mutex> lock(mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { err = std::string("CUDA error: ") + cudaGetErrorString(e); return nullptr; }
    auto it = tables.find(dev);
    if (it != tables.end()) return it->second;
    uint32_t face[26], full[26], origin;
    simple_point_masks(3, face, full, &origin);
    uint64_t* words = nullptr;
    uint32_t* d_adj = nullptr;
    const size_t bytes = ((size_t)1 << 26) / 8;
    if ((e = cudaMalloc(&words, bytes)) != cudaSuccess || (e = cudaMalloc(&d_adj, 52 * sizeof(uint32_t))) != cudaSuccess) {
        err = std::string("CUDA error: ") + cudaGetErrorString(e);
        return nullptr;
    }
    cudaMemcpy(d_adj, face, 26 * sizeof(uint32_t), cudaMemcpyHostToDevice);
    cudaMemcpy(d_adj + 26, full, 26 * sizeof(uint32_t), cudaMemcpyHostToDevice);
    e = cpmgpu::launch_table3d(words, d_adj, d_adj + 26, origin, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d_adj);
    if (e != cudaSuccess) { err = std::string("CUDA error: ") + cudaGetErrorString(e); cudaFree(words); return nullptr; }
    tables[dev] = words;
    return words;
}

// --------------------------------------------------------- DeviceSims ----
// Stream-ordered allocations (cudaMallocAsync) do not serialise the work of
// other streams the way cudaMalloc/cudaFree may; the serving loop, which
// allocates while other simulations run, asks for them.
cudaError_t DeviceSims::dev_alloc(void** p, size_t bytes) {
    return stream_ordered_ ? cudaMallocAsync(p, bytes, stream_) : cudaMalloc(p, bytes);
}
void DeviceSims::dev_free(void* p) {
    if (stream_ordered_) cudaFreeAsync(p, stream_);
    else cudaFree(p);
}

DeviceSims::~DeviceSims() {
    if (done_host_) cudaFreeHost(done_host_);
    for (auto a : aux_) cudaStreamDestroy(a);
    for (auto e : joins_) cudaEventDestroy(e);
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    for (void* p : {(void*)d_bar_, (void*)d_reg_, (void*)arena_, (void*)d_descs_, (void*)d_plans_, (void*)d_next_})
        if (p) dev_free(p);
}

namespace {
struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    }
};
}  // namespace

std::string DeviceSims::create(const std::vector<Config>& configs, const std::vector<Initial>& initials,
                               const std::vector<int>& n_samples, const std::vector<int>& n_energy,
                               bool lattice_samples, cudaStream_t stream) {
    stream_ = stream;
    // kernel attributes first: setting them later, while kernels of other
    // streams run, could wait for those kernels
    CUDA_TRY(cpmgpu::prepare_resident_kernels());
    CUDA_TRY(cpmgpu::prepare_tiled_kernels());
    // Selects the global-memory sweep for every simulation (used by the
    // tests to exercise that path on small lattices).
    force_global_ = std::getenv("CPM_GPU_FORCE_GLOBAL") != nullptr;
    // Selects the tiled sweep wherever it applies (tests use it on lattices
    // small enough for the resident sweep).
    force_tiled_ = std::getenv("CPM_GPU_FORCE_TILED") != nullptr;
    // Skips the connectivity check of every attempt, on the global-memory
    // sweep (the exact-Boltzmann test; never set in production).
    no_connectivity_ = std::getenv("CPM_GPU_TEST_NO_CONNECTIVITY") != nullptr;
    no_skip_ = std::getenv("CPM_GPU_NO_SKIP") != nullptr;
    prefer_tiled_ = std::getenv("CPM_GPU_PREFER_TILED") != nullptr;
    const size_t N = configs.size();
    layouts_.resize(N);
    descs_.resize(N);
    uint32_t t2[8];
    table2d(t2);
    bool need_t3 = false;
    // ---- sizes
    struct Offs { size_t sigma, adh, vol, itf, sp, so, slots, stats, J, lv, li, tv, ti, vt, it, dj, vt32, it32, vt32lo, it32lo, dj32, J32, la, ma, birth, energy, svol, sitf, ssp, sso, slat, err; };
    std::vector<int> tab_n(N);
    std::vector<Offs> offs(N);
    Carve cv;
    for (size_t i = 0; i < N; ++i) {
        const Config& c = configs[i];
        SimLayout& L = layouts_[i];
        L.g.init(c);
        if (L.g.n_padded >= ((int64_t)1 << 31)) return "lattice too large for the device engine (padded sites must be < 2^31)";
        L.NE = energy_count(c.D, c.energy_nbh);
        L.n_cells = (int)initials[i].type_of.size();
        L.n_samples = n_samples[i];
        L.n_energy = n_energy[i];
        L.lattice_samples = lattice_samples;
        if (c.D == 3) need_t3 = true;
        const size_t n1 = (size_t)L.n_cells + 1, nt = c.types.size(), D = (size_t)c.D;
        Offs& o = offs[i];
        o.sigma = cv.take(L.g.n_padded * 4);
        o.adh = cv.take(n1 * 2);
        o.vol = cv.take(n1 * 4);
        o.itf = cv.take(n1 * 4);
        o.sp = cv.take(n1 * D * 8);
        o.so = cv.take(n1 * D * D * 8);
        o.slots = cv.take(n1 * 8);
        o.stats = cv.take(CPM_STAT_COUNT * 8);
        o.J = cv.take((nt + 1) * (nt + 1) * 8);
        o.lv = cv.take(nt * 8);
        o.li = cv.take(nt * 8);
        o.tv = cv.take(nt * 4);
        o.ti = cv.take(nt * 4);
        uint32_t tmax = 0;
        for (auto& t : c.types) tmax = std::max({tmax, t.target_volume, t.target_interface});
        tab_n[i] = (int)std::min<uint64_t>(8192, 2 * (uint64_t)tmax + 128);
        o.vt = cv.take(nt * (size_t)tab_n[i] * 8);
        o.it = cv.take(nt * (size_t)tab_n[i] * 8);
        o.dj = cv.take((nt + 1) * (nt + 1) * (nt + 1) * 8);
        o.vt32 = cv.take(nt * (size_t)tab_n[i] * 4);
        o.it32 = cv.take(nt * (size_t)tab_n[i] * 4);
        o.vt32lo = cv.take(nt * (size_t)tab_n[i] * 4);
        o.it32lo = cv.take(nt * (size_t)tab_n[i] * 4);
        o.dj32 = cv.take((nt + 1) * (nt + 1) * (nt + 1) * 4);
        o.J32 = cv.take((nt + 1) * (nt + 1) * 4);
        // Act term: per-type parameters and the per-site acquisition MCS (zero)
        o.la = c.active.act ? cv.take(nt * 8) : 0;
        o.ma = c.active.act ? cv.take(nt * 4) : 0;
        o.birth = c.active.act ? cv.take((size_t)L.g.n_padded * 4) : 0;
        o.err = cv.take(8);
    }
    // run-window outputs after every input: the device writes them, so they
    // are neither staged on the host nor uploaded
    const size_t in_bytes = cv.off;
    for (size_t i = 0; i < N; ++i) {
        const SimLayout& L = layouts_[i];
        Offs& o = offs[i];
        const size_t n1 = (size_t)L.n_cells + 1, D = (size_t)L.g.D;
        o.energy = cv.take((size_t)std::max(1, L.n_energy) * 8);
        o.svol = cv.take((size_t)L.n_samples * n1 * 4);
        o.sitf = cv.take((size_t)L.n_samples * n1 * 4);
        o.ssp = cv.take((size_t)L.n_samples * n1 * D * 8);
        o.sso = cv.take((size_t)L.n_samples * n1 * D * D * 8);
        o.slat = lattice_samples ? cv.take((size_t)L.n_samples * L.g.n_sites * 4) : 0;
    }
    const uint64_t* t3 = nullptr;
    if (need_t3) {
        std::string err;
        t3 = device_table3d(err);
        if (!t3) return err;
    }
    CUDA_TRY(dev_alloc((void**)&arena_, std::max<size_t>(cv.off, 256)));
    CUDA_TRY(dev_alloc((void**)&d_descs_, std::max<size_t>(N, 1) * sizeof(SimDesc)));
    CUDA_TRY(dev_alloc((void**)&d_next_, sizeof(int) * 64));
    uint32_t* done_dev = nullptr;
    if (track_done_) {
        CUDA_TRY(cudaHostAlloc((void**)&done_host_, std::max<size_t>(N, 1) * 4, cudaHostAllocMapped));
        std::memset(done_host_, 0, std::max<size_t>(N, 1) * 4);
        CUDA_TRY(cudaHostGetDevicePointer((void**)&done_dev, done_host_, 0));
    }
    device_bytes_ = std::max<size_t>(cv.off, 256) + std::max<size_t>(N, 1) * sizeof(SimDesc) + sizeof(int) * 64;
    (void)t3;
    // ---- host staging, then one upload per buffer
    std::vector<char> stage(in_bytes, 0);
    // each simulation stages into its own region of `stage` and its own
    // descriptor: host threads over simulations
    auto stage_one = [&](size_t i) {
        const Config& c = configs[i];
        const SimLayout& L = layouts_[i];
        const Offs& o = offs[i];
        const size_t n1 = (size_t)L.n_cells + 1, nt = c.types.size();
        std::vector<uint32_t> padded = pad_lattice(L.g, initials[i].lattice);
        std::memcpy(stage.data() + o.sigma, padded.data(), padded.size() * 4);
        std::vector<uint16_t> adh(n1, 0);
        for (size_t id = 1; id < n1; ++id) adh[id] = (uint16_t)(initials[i].type_of[id - 1] + 1);
        std::memcpy(stage.data() + o.adh, adh.data(), n1 * 2);
        // V, I and the position sums stay zero here: launch_derive computes
        // them on the device from the uploaded lattice
        std::memset(stage.data() + o.slots, 0xFF, n1 * 8);
        std::vector<double> J((nt + 1) * (nt + 1));
        for (size_t a = 0; a <= nt; ++a)
            for (size_t b = 0; b <= nt; ++b) J[a * (nt + 1) + b] = c.adhesion[a][b];
        std::memcpy(stage.data() + o.J, J.data(), J.size() * 8);
        for (size_t t = 0; t < nt; ++t) {
            const double lv = c.types[t].lambda_volume, li = c.types[t].lambda_interface;
            std::memcpy(stage.data() + o.lv + t * 8, &lv, 8);
            std::memcpy(stage.data() + o.li + t * 8, &li, 8);
            std::memcpy(stage.data() + o.tv + t * 4, &c.types[t].target_volume, 4);
            std::memcpy(stage.data() + o.ti + t * 4, &c.types[t].target_interface, 4);
            if (c.active.act) {
                std::memcpy(stage.data() + o.la + t * 8, &c.types[t].lambda_act, 8);
                std::memcpy(stage.data() + o.ma + t * 4, &c.types[t].max_act, 4);
            }
        }
        // Exact term tables: the device adds these values where it would
        // otherwise compute lambda * ((x - target) * (x - target)) and
        // J[g][k] - J[l][k]; -ffp-contract=off keeps every operation a
        // separately rounded f64 operation, as on the device.
        {
            const int tn = tab_n[i];
            std::vector<double> vt(nt * (size_t)tn), it(nt * (size_t)tn);
            for (size_t t = 0; t < nt; ++t) {
                const double lv = c.types[t].lambda_volume, li = c.types[t].lambda_interface;
                const double tv = (double)c.types[t].target_volume, ti = (double)c.types[t].target_interface;
                for (int x = 0; x < tn; ++x) {
                    const double dv = (double)x - tv, di = (double)x - ti;
                    vt[t * tn + x] = lv * (dv * dv);
                    it[t * tn + x] = li * (di * di);
                }
            }
            std::memcpy(stage.data() + o.vt, vt.data(), vt.size() * 8);
            std::memcpy(stage.data() + o.it, it.data(), it.size() * 8);
            const size_t n1t = nt + 1;
            std::vector<double> dj(n1t * n1t * n1t);
            for (size_t l = 0; l < n1t; ++l)
                for (size_t g = 0; g < n1t; ++g)
                    for (size_t k = 0; k < n1t; ++k) dj[(l * n1t + g) * n1t + k] = J[g * n1t + k] - J[l * n1t + k];
            std::memcpy(stage.data() + o.dj, dj.data(), dj.size() * 8);
            // float copies (round to nearest) for the bounded pre-decision
            auto put32 = [&](size_t off, const std::vector<double>& v) {
                std::vector<float> f(v.size());
                for (size_t q = 0; q < v.size(); ++q) f[q] = (float)v[q];
                std::memcpy(stage.data() + off, f.data(), f.size() * 4);
            };
            put32(o.vt32, vt);
            put32(o.it32, it);
            auto put32lo = [&](size_t off, const std::vector<double>& v) {
                std::vector<float> f(v.size());
                for (size_t q = 0; q < v.size(); ++q) f[q] = (float)(v[q] - (double)(float)v[q]);
                std::memcpy(stage.data() + off, f.data(), f.size() * 4);
            };
            put32lo(o.vt32lo, vt);
            put32lo(o.it32lo, it);
            put32(o.dj32, dj);
            put32(o.J32, J);
        }
        // descriptor
        SimDesc& s = descs_[i];
        std::memset(&s, 0, sizeof s);
        s.D = c.D;
        s.periodic = c.periodic;
        for (int d = 0; d < 3; ++d) {
            s.dims[d] = (int32_t)L.g.dims[d];
            s.pdims[d] = (int32_t)L.g.pdims[d];
            s.strides[d] = L.g.strides[d];
        }
        s.n_sites = L.g.n_sites;
        s.n_padded = L.g.n_padded;
        s.no_connectivity = no_connectivity_ ? 1 : 0;
        s.sweep_flags = no_skip_ ? 1 : 0;
        s.n_colors = 1;
        s.max_class = 1;
        for (int d = 0; d < 3; ++d) {
            if (d >= c.D) { s.ncol[d] = 1; s.lim[d] = 1; continue; }
            const int64_t Ld = L.g.dims[d];
            if (Ld == 1) { s.ncol[d] = 1; s.lim[d] = 1; }
            else if (c.periodic && (Ld & 1)) { s.ncol[d] = 3; s.lim[d] = (int32_t)(Ld - 1); }
            else { s.ncol[d] = 2; s.lim[d] = (int32_t)Ld; }
            s.n_colors *= s.ncol[d];
            s.max_class *= (int32_t)((s.lim[d] + 1) / 2);
        }
        auto cs = stencil(NBH_VON_NEUMANN, c.D);
        s.n_copy = (int)cs.size();
        for (size_t k = 0; k < cs.size(); ++k) {
            s.copy_off[k] = cs[k][0] * L.g.strides[0] + cs[k][1] * L.g.strides[1] + cs[k][2] * L.g.strides[2];
            for (int d = 0; d < 3; ++d) s.copy_vec[k][d] = (int8_t)cs[k][d];
        }
        auto es = stencil(c.energy_nbh, c.D);
        s.n_energy = (int)es.size();
        s.energy_pos_mask = 0;
        for (size_t k = 0; k < es.size(); ++k) {
            s.energy_off[k] = es[k][0] * L.g.strides[0] + es[k][1] * L.g.strides[1] + es[k][2] * L.g.strides[2];
            for (int d = 0; d < 3; ++d) s.energy_vec[k][d] = (int8_t)es[k][d];
            for (int d = 0; d < c.D; ++d) {
                if (es[k][d] > 0) { s.energy_pos_mask |= 1u << k; break; }
                if (es[k][d] < 0) break;
            }
        }
        auto ts = stencil(c.D == 2 ? NBH_MOORE : NBH_TWENTY_SIX, c.D);
        for (size_t k = 0; k < ts.size(); ++k) {
            s.topo_off[k] = ts[k][0] * L.g.strides[0] + ts[k][1] * L.g.strides[1] + ts[k][2] * L.g.strides[2];
            for (int d = 0; d < 3; ++d) s.topo_vec[k][d] = (int8_t)ts[k][d];
        }
        std::memcpy(s.table2d, t2, sizeof t2);
        s.n_types = (int)nt;
        s.min_cell_volume = c.min_cell_volume;
        s.seed = c.seed;
        s.n_cells = L.n_cells;
        char* base = arena_;
        s.sigma = (uint32_t*)(base + o.sigma);
        s.adh_of = (const uint16_t*)(base + o.adh);
        s.acceptance = c.acceptance == ACC_METROPOLIS ? 0 : 1;
        s.act = c.active.act ? 1 : 0;
        s.lambda_act = c.active.act ? (const double*)(base + o.la) : nullptr;
        s.max_act = c.active.act ? (const uint32_t*)(base + o.ma) : nullptr;
        s.birth = c.active.act ? (uint32_t*)(base + o.birth) : nullptr;
        s.volume = (uint32_t*)(base + o.vol);
        s.interface = (uint32_t*)(base + o.itf);
        s.sum_pos = (int64_t*)(base + o.sp);
        s.sum_outer = (int64_t*)(base + o.so);
        s.slots = (unsigned long long*)(base + o.slots);
        s.stats = (unsigned long long*)(base + o.stats);
        s.J = (const double*)(base + o.J);
        s.lambda_v = (const double*)(base + o.lv);
        s.lambda_i = (const double*)(base + o.li);
        s.target_v = (const uint32_t*)(base + o.tv);
        s.target_i = (const uint32_t*)(base + o.ti);
        s.vterm = (const double*)(base + o.vt);
        s.iterm = (const double*)(base + o.it);
        s.dj = (const double*)(base + o.dj);
        s.vterm32 = (const float*)(base + o.vt32);
        s.iterm32 = (const float*)(base + o.it32);
        s.vterm32lo = (const float*)(base + o.vt32lo);
        s.iterm32lo = (const float*)(base + o.it32lo);
        s.dj32 = (const float*)(base + o.dj32);
        s.J32 = (const float*)(base + o.J32);
        s.tab_n = tab_n[i];
        s.mcs = 0;
        s.energy_out = (double*)(base + o.energy);
        s.sample_volume = (uint32_t*)(base + o.svol);
        s.sample_interface = (uint32_t*)(base + o.sitf);
        s.sample_sum_pos = (int64_t*)(base + o.ssp);
        s.sample_sum_outer = (int64_t*)(base + o.sso);
        s.sample_lattice = lattice_samples ? (uint32_t*)(base + o.slat) : nullptr;
        s.error = (int32_t*)(base + o.err);
        s.done_flag = done_dev ? done_dev + i : nullptr;
    };
    {
        const unsigned nthreads =
            (unsigned)std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), N));
        if (nthreads <= 1 || N < 8) {
            for (size_t i = 0; i < N; ++i) stage_one(i);
        } else {
            std::atomic<size_t> next{0};
            std::vector<std::thread> th;
            for (unsigned t = 0; t < nthreads; ++t)
                th.emplace_back([&] {
                    for (size_t i; (i = next.fetch_add(1)) < N;) stage_one(i);
                });
            for (auto& t : th) t.join();
        }
    }
    h2d_bytes_ += in_bytes + N * sizeof(SimDesc);
    CUDA_TRY(cudaMemcpyAsync(arena_, stage.data(), in_bytes, cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(d_descs_, descs_.data(), N * sizeof(SimDesc), cudaMemcpyHostToDevice, stream_));
    // the derived state of every fresh lattice (initialization.rs:396-436)
    {
        int64_t max_sites = 1;
        for (const SimLayout& L : layouts_) max_sites = std::max<int64_t>(max_sites, L.g.n_sites);
        CUDA_TRY(cpmgpu::launch_derive(d_descs_, (int)N, max_sites, stream_));
    }
    CUDA_TRY(cudaStreamSynchronize(stream_));
    return "";
}

DeviceSims::Path DeviceSims::path(size_t i) const {
    const SimLayout& L = layouts_[i];
    if (force_global_ || no_connectivity_) return GLOBAL;
    // Metropolis-Hastings acceptance and the Act term run on the same
    // sweeps as Metropolis, in kernel variants of their own
    int dims[3] = {(int)L.g.dims[0], (int)L.g.dims[1], (int)L.g.dims[2]}, nt[3] = {1, 1, 1}, max_box = 0;
    const bool tiled_ok = cpmgpu::tiled_plan(L.g.D, dims, L.g.periodic, nt, &max_box) &&
                          cpmgpu::tiled_smem_bytes(max_box, L.n_cells, 0, L.g.D, 0) <= cpmgpu::resident_smem_limit();
    // the resident sweep keeps cell ids in 16 bits
    if (!force_tiled_ && L.n_cells < 65535 &&
        cpmgpu::resident_smem_bytes(L.g.n_padded, L.n_cells) <= cpmgpu::resident_smem_limit()) {
        // The path is a function of the simulation's own configuration, so a
        // simulation's trajectory is the same alone and inside any batch.
        // CPM_GPU_PREFER_TILED opts a simulation with at least 8 tiles per
        // colour into the tiled sweep (many SMs instead of one; a different,
        // equally exact chain, hence opt-in).
        const int per_color = (nt[0] * nt[1] * nt[2]) >> L.g.D;
        if (prefer_tiled_ && tiled_ok && per_color >= 8) return TILED;
        return RESIDENT;
    }
    return tiled_ok ? TILED : GLOBAL;
}

// ------------------------------------------------------ grid tuner ----
// The tiled sweep's grid (how many CTAs share the tiles of a colour) is the
// one launch parameter the trajectory does not depend on: tiles, claims and
// priorities are functions of (seed, MCS, tile id). The tuner times it on
// the simulation's own first MCS: while a shape has no choice yet, the run
// starts with short trial launches of each candidate grid (one, two, three
// and four tiles per CTA), each twice, bracketed by CUDA events; then it
// waits for them, keeps the fastest per MCS for the rest of the run and for
// every later run of the same shape in the process. The trials are MCS the
// run performs anyway, so tuning changes no result.
namespace {
struct TuneEntry {
    std::vector<int> cand;
    std::vector<double> us_per_mcs;  // best measurement per candidate
    int chosen = 0;
    bool done = false;
};
std::mutex g_tune_mu;
std::map<std::array<int, 9>, TuneEntry>& tune_table() {
    static std::map<std::array<int, 9>, TuneEntry> t;
    return t;
}
}  // namespace

std::string tuning_report() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::string o = "[";
    bool first = true;
    for (auto& kv : tune_table()) {
        const auto& k = kv.first;
        const TuneEntry& e = kv.second;
        if (!first) o += ",";
        first = false;
        o += "{\"dim\":" + std::to_string(k[0]) + ",\"energy_neighbours\":" + std::to_string(k[1]) +
             ",\"odd\":" + std::to_string(k[2]) + ",\"modes\":" + std::to_string(k[3]) + ",\"tiles_per_axis\":[" +
             std::to_string(k[4]) + "," + std::to_string(k[5]) + "," + std::to_string(k[6]) +
             "],\"tiles_per_colour\":" + std::to_string(k[7]) +
             ",\"done\":" + (e.done ? "true" : "false") + ",\"grid\":" + std::to_string(e.chosen) +
             ",\"candidates\":[";
        for (size_t i = 0; i < e.cand.size(); ++i) {
            // untimed candidates (a shape whose runs were too short for the
            // trials) report -1
            const double us = i < e.us_per_mcs.size() && e.us_per_mcs[i] < 1e200 ? e.us_per_mcs[i] : -1.0;
            char b[96];
            std::snprintf(b, sizeof b, "%s[%d,%.3f]", i ? "," : "", e.cand[i], us);
            o += b;
        }
        o += "]}";
    }
    return o + "]";
}

// One simulation on the tiled sweep: the run window is replayed from the
// host, one cooperative launch per chunk plus energy and sample launches.
std::string DeviceSims::run_tiled(const RunPlan& p, const uint64_t* t3) {
    const SimLayout& L = layouts_[p.sim];
    int dims[3] = {(int)L.g.dims[0], (int)L.g.dims[1], (int)L.g.dims[2]}, nt[3], max_box = 0;
    cpmgpu::tiled_plan(L.g.D, dims, L.g.periodic, nt, &max_box);
    // the cell registry in shared memory if it fits beside all the box's
    // position sums (else in HBM), position sums of up to 1024 listed cells
    // per box in shared memory (as many as fit), then the energy tables if
    // they fit beside the tile state
    const size_t lim = cpmgpu::resident_smem_limit();
    int cl_cap = (int)std::min<int64_t>(std::min<int64_t>(max_box, L.n_cells), 1024);
    const int reg_smem = cpmgpu::tiled_smem_bytes(max_box, L.n_cells, cl_cap, L.g.D, 1) <= lim ? 1 : 0;
    while (cl_cap > 0 && cpmgpu::tiled_smem_bytes(max_box, L.n_cells, cl_cap, L.g.D, reg_smem) > lim) cl_cap /= 2;
    size_t smem = cpmgpu::tiled_smem_bytes(max_box, L.n_cells, cl_cap, L.g.D, reg_smem);
    const size_t tab = cpmgpu::tiled_table_bytes(descs_[p.sim].n_types, descs_[p.sim].tab_n);
    const int tables_in_smem = smem + tab <= lim;
    if (tables_in_smem) smem += tab;
    int per_sm = 0, dev = 0, sms = 1;
    int odd = 0;
    for (int d = 0; d < L.g.D; ++d) odd |= L.g.periodic && (L.g.dims[d] & 1);
    const int modes = descs_[p.sim].acceptance || descs_[p.sim].act ? 1 : 0;
    CUDA_TRY(cpmgpu::tiled_occupancy(L.g.D, L.NE, odd, modes, smem, &per_sm));
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int tiles = 1;
    for (int d = 0; d < L.g.D; ++d) tiles *= nt[d];
    int grid = std::max(1, std::min(tiles >> L.g.D, std::max(1, per_sm) * sms));
    // CPM_GPU_TILED_GRID caps the grid (several tiles per CTA); the tiling,
    // and so the trajectory, does not depend on it
    const char* grid_env = std::getenv("CPM_GPU_TILED_GRID");
    if (grid_env) grid = std::max(1, std::min(grid, std::atoi(grid_env)));
    if (tiled_grid_cap_ > 0) grid = std::max(1, std::min(grid, tiled_grid_cap_));
    if ((tiles >> L.g.D) > 511 * grid) return "tiled sweep: too many tiles per CTA for this lattice";
    // the tuner's entry for this shape (none when the grid is set from
    // outside: the environment, a serving cap, or CPM_GPU_NO_TUNE)
    const int per_color = tiles >> L.g.D;
    const std::array<int, 9> tkey = {L.g.D, L.NE, odd, modes, nt[0], L.g.D > 1 ? nt[1] : 1, L.g.D > 2 ? nt[2] : 1,
                                     per_color, (int)smem};
    const bool tune = !grid_env && tiled_grid_cap_ <= 0 && !std::getenv("CPM_GPU_NO_TUNE");
    std::vector<int> trials;  // grids still to time in this run, in order
    if (tune) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        TuneEntry& te = tune_table()[tkey];
        if (te.cand.empty()) {
            for (int k = 1; k <= 4; ++k) {
                const int g = (per_color + k - 1) / k;
                if (g < 1 || g > grid || per_color > 511 * g) continue;
                if (std::find(te.cand.begin(), te.cand.end(), g) == te.cand.end()) te.cand.push_back(g);
            }
            te.us_per_mcs.assign(te.cand.size(), 1e300);
            te.chosen = grid;
        }
        if (te.done) grid = te.chosen;
        else if (te.cand.size() > 1)
            for (int rep = 0; rep < 2; ++rep) trials.insert(trials.end(), te.cand.begin(), te.cand.end());
    }
    const int grid_max = grid;  // the largest grid any launch of this run uses
    // CPM_GPU_TEST_BARRIER_TIMEOUT (tests only): the grid barrier waits for
    // one CTA more than the grid has, so every bounded wait runs out, the
    // kernel records the timeout and returns; nothing else changes
    const int barrier_extra = std::getenv("CPM_GPU_TEST_BARRIER_TIMEOUT") ? 1 : 0;
    if (!d_bar_) CUDA_TRY(dev_alloc(&d_bar_, 64));
    // each CTA's cell registry in HBM (when it is not in shared memory): a
    // stamp and a box slot per cell id
    const size_t reg = reg_smem ? 0 : 2 * (size_t)grid_max * (size_t)(L.n_cells + 1) * 4;
    if (reg > reg_cap_) {
        if (d_reg_) dev_free(d_reg_);
        d_reg_ = nullptr;
        reg_cap_ = 0;
        CUDA_TRY(dev_alloc((void**)&d_reg_, reg));
        reg_cap_ = reg;
        device_bytes_ += reg;
    }
    SimDesc* d_sim = d_descs_ + p.sim;
    unsigned long long* claims = descs_[p.sim].slots;
    auto launch = [&](uint64_t m, int g) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(d_bar_, 0, 64, stream_);
        if (e == cudaSuccess)
            e = cpmgpu::launch_tiled(L.g.D, L.NE, odd, modes, d_sim, m, nt, d_bar_, claims, reg_smem ? nullptr : d_reg_, t3,
                                     max_box, tables_in_smem, barrier_extra, cl_cap, reg_smem, smem, g, stream_,
                                     L.n_cells);
        return e;
    };
    // trial launches of TRIAL_MCS each (3D MCS cost more: fewer)
    const uint64_t TRIAL_MCS = L.g.D == 2 ? 8 : 4;
    auto chunk = [&](uint64_t n) -> std::string {
        if (!trials.empty() && n >= TRIAL_MCS * trials.size() + 1) {
            std::vector<cudaEvent_t> ev(trials.size() + 1);
            for (auto& x : ev) CUDA_TRY(cudaEventCreate(&x));
            CUDA_TRY(cudaEventRecord(ev[0], stream_));
            for (size_t i = 0; i < trials.size(); ++i) {
                CUDA_TRY(launch(TRIAL_MCS, trials[i]));
                CUDA_TRY(cudaEventRecord(ev[i + 1], stream_));
            }
            n -= TRIAL_MCS * trials.size();
            CUDA_TRY(cudaEventSynchronize(ev.back()));
            {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                TuneEntry& te = tune_table()[tkey];
                for (size_t i = 0; i < trials.size(); ++i) {
                    float ms = 0.f;
                    CUDA_TRY(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
                    const size_t c = std::find(te.cand.begin(), te.cand.end(), trials[i]) - te.cand.begin();
                    te.us_per_mcs[c] = std::min(te.us_per_mcs[c], 1000.0 * ms / (double)TRIAL_MCS);
                }
                size_t best = 0;
                for (size_t c = 1; c < te.cand.size(); ++c)
                    if (te.us_per_mcs[c] < te.us_per_mcs[best]) best = c;
                te.chosen = te.cand[best];
                te.done = true;
                grid = te.chosen;
            }
            for (auto& x : ev) cudaEventDestroy(x);
            trials.clear();
        }
        // at most 2^18 MCS per launch: the barrier counter (32 bits) grows by
        // grid x 2 x colours per MCS within a launch
        while (n > 0) {
            const uint64_t m = std::min<uint64_t>(n, 1ull << 18);
            CUDA_TRY(launch(m, grid));
            n -= m;
        }
        return "";
    };
    std::string e;
    uint64_t burned = 0;
    int e_idx = 0;
    while (burned < p.burn_in) {
        const uint64_t c = std::min(p.interval, p.burn_in - burned);
        if (!(e = chunk(c)).empty()) return e;
        burned += c;
        if (burned >= p.energy_sample_start) {
            if (descs_[p.sim].energy_out && e_idx < L.n_energy)
                CUDA_TRY(cpmgpu::launch_energy(L.g.D, L.NE, d_sim, descs_[p.sim].energy_out + e_idx, stream_));
            ++e_idx;
        }
    }
    for (int smp = 0; smp < p.n_samples; ++smp) {
        if (!(e = chunk(p.interval)).empty()) return e;
        if (descs_[p.sim].energy_out && e_idx + smp < L.n_energy)
            CUDA_TRY(cpmgpu::launch_energy(L.g.D, L.NE, d_sim, descs_[p.sim].energy_out + e_idx + smp, stream_));
        if (p.write_samples)
            CUDA_TRY(cpmgpu::launch_sample(L.g.D, d_sim, smp, p.write_lattice, L.g.n_sites, stream_));
    }
    tiled_ran_.push_back(p.sim);
    return "";
}

std::string DeviceSims::run(const std::vector<RunPlan>& plans, int grid_override) {
    std::string err;
    const uint64_t* t3 = nullptr;
    // group plans by kernel: (path, D, NE); resident plans also by block
    // variant (0: 512 threads, 1: 256); tiled plans run one by one
    std::map<std::tuple<int, int, int>, std::vector<RunPlan>> groups;
    std::vector<RunPlan> tiled;
    for (const RunPlan& p : plans) {
        const SimLayout& L = layouts_[p.sim];
        if (L.g.D == 3 && !t3) {
            t3 = device_table3d(err);
            if (!t3) return err;
        }
        const Path pa = path(p.sim);
        if (pa == TILED) { tiled.push_back(p); continue; }
        // 0: global sweep; resident: 1 + variant, + 2 with Metropolis-Hastings or Act
        const int modes = descs_[p.sim].acceptance || descs_[p.sim].act ? 1 : 0;
        const int kind = pa == RESIDENT ? 1 + cpmgpu::resident_variant(L.g.n_padded, L.n_cells) + 2 * modes : 0;
        groups[std::make_tuple(kind, L.g.D, L.NE)].push_back(p);
    }
    for (const RunPlan& p : tiled) {
        err = run_tiled(p, t3);
        if (!err.empty()) return err;
    }
    if (groups.empty()) return "";
    if (groups.size() > 64) return "too many kinds of simulation in one run (more than 64 kernel groups)";
    size_t total = 0;
    for (auto& kv : groups) total += kv.second.size();
    if (total > plans_cap_) {
        if (d_plans_) dev_free(d_plans_);
        d_plans_ = nullptr;
        CUDA_TRY(dev_alloc((void**)&d_plans_, total * sizeof(RunPlan)));
        plans_cap_ = total;
    }
    std::vector<RunPlan> flat;
    std::vector<std::pair<size_t, size_t>> ranges;
    for (auto& kv : groups) {
        // largest simulations first: better tail behaviour of the persistent queue
        std::sort(kv.second.begin(), kv.second.end(), [&](const RunPlan& a, const RunPlan& b) {
            return layouts_[a.sim].g.n_sites > layouts_[b.sim].g.n_sites;
        });
        ranges.push_back({flat.size(), kv.second.size()});
        flat.insert(flat.end(), kv.second.begin(), kv.second.end());
    }
    CUDA_TRY(cudaMemcpyAsync(d_plans_, flat.data(), flat.size() * sizeof(RunPlan), cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaMemsetAsync(d_next_, 0, sizeof(int) * 64, stream_));
    int dev = 0, sms = 1;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // groups after the first run on auxiliary streams forked from and joined
    // to the object's stream, so one group's CTAs start as another's drain
    if (groups.size() > 1 && aux_.empty()) {
        aux_.resize(std::min<size_t>(groups.size(), 16) - 1);
        for (auto& a : aux_) CUDA_TRY(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
        joins_.resize(aux_.size());
        for (auto& e : joins_) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (groups.size() > 1) CUDA_TRY(cudaEventRecord(ev_fork_, stream_));
    size_t gi = 0;
    for (auto& kv : groups) {
        const auto r = ranges[gi];
        cudaStream_t gst = stream_;
        if (gi > 0 && gi - 1 < aux_.size()) {
            gst = aux_[gi - 1];
            CUDA_TRY(cudaStreamWaitEvent(gst, ev_fork_, 0));
        }
        const int res = std::get<0>(kv.first), D = std::get<1>(kv.first), NE = std::get<2>(kv.first);
        int max_cells = 0;
        size_t smem = 0;
        for (size_t k = 0; k < r.second; ++k) {
            const SimLayout& L = layouts_[flat[r.first + k].sim];
            max_cells = std::max(max_cells, L.n_cells);
            smem = std::max(smem, cpmgpu::resident_smem_bytes(L.g.n_padded, L.n_cells));
        }
        if (res) {
            const int variant = (res - 1) & 1, modes = (res - 1) >> 1;
            int per_sm = 1;
            CUDA_TRY(cpmgpu::resident_occupancy(D, NE, variant, modes, smem, &per_sm));
            int grid = grid_override > 0 ? grid_override : std::min<int>((int)r.second, sms * std::max(1, per_sm));
            CUDA_TRY(cpmgpu::launch_resident(D, NE, variant, modes, d_descs_, d_plans_ + r.first, (int)r.second, d_next_ + gi, t3, smem,
                                             std::max(1, grid), gst));
        } else {
            int grid = grid_override > 0 ? grid_override : std::min<int>((int)r.second, sms * 4);
            CUDA_TRY(cpmgpu::launch_sweep(D, NE, d_descs_, d_plans_ + r.first, (int)r.second, d_next_ + gi, t3, max_cells,
                                          std::max(1, grid), gst));
        }
        if (gst != stream_) {
            CUDA_TRY(cudaEventRecord(joins_[gi - 1], gst));
            CUDA_TRY(cudaStreamWaitEvent(stream_, joins_[gi - 1], 0));
        }
        ++gi;
    }
    return "";
}

std::string DeviceSims::sync() {
    CUDA_TRY(cudaStreamSynchronize(stream_));
    // bounded device waits record a timeout instead of hanging
    for (size_t i : tiled_ran_) {
        int32_t err = 0;
        CUDA_TRY(cudaMemcpy(&err, descs_[i].error, 4, cudaMemcpyDeviceToHost));
        if (err) return "device wait timed out in the tiled sweep (error " + std::to_string(err) + ")";
    }
    tiled_ran_.clear();
    return "";
}

std::string DeviceSims::read_padded(size_t i, std::vector<uint32_t>& out) const {
    out.resize((size_t)layouts_[i].g.n_padded);
    d2h_bytes_ += out.size() * 4;
    CUDA_TRY(cudaMemcpy(out.data(), descs_[i].sigma, out.size() * 4, cudaMemcpyDeviceToHost));
    return "";
}

std::string DeviceSims::read_cells(size_t i, std::vector<uint32_t>& vol, std::vector<uint32_t>& itf,
                                   std::vector<int64_t>& sp, std::vector<int64_t>& so) const {
    const size_t n1 = layouts_[i].n_cells + 1, D = layouts_[i].g.D;
    vol.resize(n1); itf.resize(n1); sp.resize(n1 * D); so.resize(n1 * D * D);
    d2h_bytes_ += n1 * 4;
    CUDA_TRY(cudaMemcpy(vol.data(), descs_[i].volume, n1 * 4, cudaMemcpyDeviceToHost));
    d2h_bytes_ += n1 * 4;
    CUDA_TRY(cudaMemcpy(itf.data(), descs_[i].interface, n1 * 4, cudaMemcpyDeviceToHost));
    d2h_bytes_ += sp.size() * 8;
    CUDA_TRY(cudaMemcpy(sp.data(), descs_[i].sum_pos, sp.size() * 8, cudaMemcpyDeviceToHost));
    d2h_bytes_ += so.size() * 8;
    CUDA_TRY(cudaMemcpy(so.data(), descs_[i].sum_outer, so.size() * 8, cudaMemcpyDeviceToHost));
    return "";
}

std::string DeviceSims::set_desc(size_t i, const SimDesc& d) {
    descs_[i] = d;
    CUDA_TRY(cudaMemcpyAsync(d_descs_ + i, &descs_[i], sizeof(SimDesc), cudaMemcpyHostToDevice, stream_));
    return "";
}

std::string DeviceSims::read_energy(size_t i, std::vector<double>& e) const {
    e.resize(layouts_[i].n_energy);
    if (!e.empty()) { d2h_bytes_ += e.size() * 8; CUDA_TRY(cudaMemcpy(e.data(), descs_[i].energy_out, e.size() * 8, cudaMemcpyDeviceToHost)); }
    return "";
}

std::string DeviceSims::read_samples(size_t i, int n, std::vector<uint32_t>& vol, std::vector<uint32_t>& itf,
                                     std::vector<int64_t>& sp, std::vector<int64_t>& so,
                                     std::vector<uint32_t>* lattice) const {
    const size_t n1 = layouts_[i].n_cells + 1, D = layouts_[i].g.D;
    vol.resize(n * n1); itf.resize(n * n1); sp.resize(n * n1 * D); so.resize(n * n1 * D * D);
    if (n == 0) return "";
    d2h_bytes_ += vol.size() * 4;
    CUDA_TRY(cudaMemcpy(vol.data(), descs_[i].sample_volume, vol.size() * 4, cudaMemcpyDeviceToHost));
    d2h_bytes_ += itf.size() * 4;
    CUDA_TRY(cudaMemcpy(itf.data(), descs_[i].sample_interface, itf.size() * 4, cudaMemcpyDeviceToHost));
    d2h_bytes_ += sp.size() * 8;
    CUDA_TRY(cudaMemcpy(sp.data(), descs_[i].sample_sum_pos, sp.size() * 8, cudaMemcpyDeviceToHost));
    d2h_bytes_ += so.size() * 8;
    CUDA_TRY(cudaMemcpy(so.data(), descs_[i].sample_sum_outer, so.size() * 8, cudaMemcpyDeviceToHost));
    if (lattice && descs_[i].sample_lattice) {
        lattice->resize((size_t)n * layouts_[i].g.n_sites);
        d2h_bytes_ += lattice->size() * 4;
        CUDA_TRY(cudaMemcpy(lattice->data(), descs_[i].sample_lattice, lattice->size() * 4, cudaMemcpyDeviceToHost));
    }
    return "";
}

std::string DeviceSims::read_stats(size_t i, std::vector<uint64_t>& stats) const {
    stats.resize(CPM_STAT_COUNT);
    d2h_bytes_ += CPM_STAT_COUNT * 8;
    CUDA_TRY(cudaMemcpy(stats.data(), descs_[i].stats, CPM_STAT_COUNT * 8, cudaMemcpyDeviceToHost));
    return "";
}

std::string DeviceSims::write_act_state(size_t i, const std::vector<uint32_t>* birth, uint64_t mcs) {
    if (birth) {
        if (!descs_[i].birth) return "write_act_state: the Act term is not active";
        if (birth->size() != (size_t)layouts_[i].g.n_padded) return "write_act_state: size mismatch";
        h2d_bytes_ += birth->size() * 4;
        CUDA_TRY(cudaMemcpy(descs_[i].birth, birth->data(), birth->size() * 4, cudaMemcpyHostToDevice));
    }
    descs_[i].mcs = mcs;
    CUDA_TRY(cudaMemcpy(&d_descs_[i].mcs, &mcs, 8, cudaMemcpyHostToDevice));
    return "";
}

std::string DeviceSims::read_birth(size_t i, std::vector<uint32_t>& birth) const {
    if (!descs_[i].birth) return "read_birth: the Act term is not active";
    birth.resize((size_t)layouts_[i].g.n_padded);
    d2h_bytes_ += birth.size() * 4;
    CUDA_TRY(cudaMemcpy(birth.data(), descs_[i].birth, birth.size() * 4, cudaMemcpyDeviceToHost));
    return "";
}

std::string DeviceSims::read_mcs(size_t i, uint64_t& mcs) const {
    d2h_bytes_ += 8;
    CUDA_TRY(cudaMemcpy(&mcs, &d_descs_[i].mcs, 8, cudaMemcpyDeviceToHost));
    return "";
}

// ---- topology readouts on the device (cpm_readout.cu) ----
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Energy stencil of a simulation as the readout kernels take it: offsets in
// {-1,0,1}^D with at most this many nonzero components.
static int energy_maxnz(int D, int NE) {
    if (NE == 2 * D) return 1;  // von Neumann
    if (NE == 18) return 2;     // Eighteen
    return D;                   // Moore (2D), TwentySix (3D)
}

static uint64_t readout_units(int64_t n_sites, int n_cells) {
    const uint64_t n = (uint64_t)n_cells, tri = n * (n + 1) / 2, U = (uint64_t)cpmgpu::readout_unit();
    const uint64_t span = std::max<uint64_t>({(uint64_t)n_sites, tri, n + 1});
    return (span + U - 1) / U;
}

static size_t readout_scratch(int64_t n_sites, int n_cells) {
    const uint64_t n = (uint64_t)n_cells;
    return align256((size_t)n_sites * 8) + align256(n * (n + 1) / 2 * 4) + align256((n + 1) * 4);
}

size_t topology_bytes(int64_t n_sites, int n_cells) {
    // scratch, unit counters and offsets, and room for the output streams
    return readout_scratch(n_sites, n_cells) + readout_units(n_sites, n_cells) * 36 + (size_t)n_sites * 4 +
           (size_t)n_cells * 64 + 4096;
}

std::string DeviceSims::topology(const std::vector<size_t>& sims, const std::vector<int>& ns,
                                 std::vector<std::vector<Topo>>& out) {
    const size_t M = sims.size();
    out.assign(M, {});
    int max_ns = 0;
    for (size_t m = 0; m < M; ++m) {
        out[m].resize((size_t)std::max(0, ns[m]));
        max_ns = std::max(max_ns, ns[m]);
    }
    if (max_ns <= 0) return "";
    std::vector<size_t> base(M);
    std::vector<int64_t> units(M);
    size_t total = 0;
    int64_t all_units = 0;
    for (size_t m = 0; m < M; ++m) {
        const size_t i = sims[m];
        const SimLayout& L = layouts_[i];
        if (ns[m] > 0 && !descs_[i].sample_lattice) return "topology readouts need the lattice samples";
        if (L.g.n_sites >= ((int64_t)1 << 31)) return "lattice too large for the topology readouts (2^31 sites)";
        base[m] = total;
        total += readout_scratch(L.g.n_sites, L.n_cells);
        units[m] = (int64_t)readout_units(L.g.n_sites, L.n_cells);
        all_units += units[m];
    }
    struct Buf {
        DeviceSims* d;
        void* p = nullptr;
        size_t cap = 0;
        ~Buf() { if (p) d->dev_free(p); }
        cudaError_t reserve(size_t need) {
            if (need <= cap) return cudaSuccess;
            if (p) d->dev_free(p);
            p = nullptr;
            cap = 0;
            const cudaError_t e = d->dev_alloc(&p, need);
            if (e == cudaSuccess) cap = need;
            return e;
        }
    };
    Buf scratch{this}, d_items{this}, d_prefix{this}, d_cnt{this}, d_off{this}, d_pairs{this}, d_med{this},
        d_frag{this};
    CUDA_TRY(scratch.reserve(std::max<size_t>(total, 256)));
    CUDA_TRY(cudaMemsetAsync(scratch.p, 0, total, stream_));  // contact tables and component counts start at zero
    CUDA_TRY(d_items.reserve(M * sizeof(ReadoutItem)));
    CUDA_TRY(d_prefix.reserve((M + 1) * 8));
    CUDA_TRY(d_cnt.reserve((size_t)std::max<int64_t>(all_units, 1) * 12));
    CUDA_TRY(d_off.reserve((size_t)std::max<int64_t>(all_units, 1) * 24));
    std::vector<ReadoutItem> items;
    std::vector<int64_t> prefix;
    std::vector<size_t> who;
    std::vector<uint32_t> cnt, h_pairs, h_med, h_frag;
    std::vector<uint64_t> off;
    for (int s = 0; s < max_ns; ++s) {
        items.clear();
        who.clear();
        prefix.assign(1, 0);
        for (size_t m = 0; m < M; ++m) {
            if (ns[m] <= s) continue;
            const size_t i = sims[m];
            const SimLayout& L = layouts_[i];
            const uint64_t n = (uint64_t)L.n_cells, tri = n * (n + 1) / 2;
            char* b = (char*)scratch.p + base[m];
            ReadoutItem it;
            std::memset(&it, 0, sizeof it);
            it.lat = descs_[i].sample_lattice + (size_t)s * (size_t)L.g.n_sites;
            it.parent = (uint32_t*)b;
            it.aux = (uint32_t*)b + L.g.n_sites;
            it.tri = (uint32_t*)(b + align256((size_t)L.g.n_sites * 8));
            it.ncomp = (uint32_t*)(b + align256((size_t)L.g.n_sites * 8) + align256(tri * 4));
            it.n_sites = L.g.n_sites;
            it.tri_n = (int64_t)tri;
            for (int d = 0; d < 3; ++d) it.dims[d] = d < L.g.D ? (int32_t)L.g.dims[d] : 1;
            it.D = L.g.D;
            it.periodic = L.g.periodic ? 1 : 0;
            it.n_cells = L.n_cells;
            it.energy_maxnz = energy_maxnz(L.g.D, L.NE);
            items.push_back(it);
            who.push_back(m);
            prefix.push_back(prefix.back() + units[m]);
        }
        const int K = (int)items.size();
        const int64_t T = prefix.back();
        CUDA_TRY(cudaMemcpyAsync(d_items.p, items.data(), K * sizeof(ReadoutItem), cudaMemcpyHostToDevice, stream_));
        CUDA_TRY(cudaMemcpyAsync(d_prefix.p, prefix.data(), (K + 1) * 8, cudaMemcpyHostToDevice, stream_));
        CUDA_TRY(cudaMemsetAsync(d_cnt.p, 0, (size_t)T * 12, stream_));
        const ReadoutItem* di = (const ReadoutItem*)d_items.p;
        const int64_t* dp = (const int64_t*)d_prefix.p;
        for (int pass = 0; pass < 4; ++pass)
            CUDA_TRY(cpmgpu::launch_readout(pass, di, K, dp, T, (uint32_t*)d_cnt.p, nullptr, nullptr, nullptr,
                                            nullptr, stream_));
        cnt.resize((size_t)T * 3);
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), d_cnt.p, (size_t)T * 12, cudaMemcpyDeviceToHost, stream_));
        CUDA_TRY(cudaStreamSynchronize(stream_));
        off.resize((size_t)T * 3);
        uint64_t acc[3] = {0, 0, 0};
        for (int64_t u = 0; u < T; ++u)
            for (int k = 0; k < 3; ++k) {
                off[3 * u + k] = acc[k];
                acc[k] += cnt[3 * u + k];
            }
        CUDA_TRY(d_pairs.reserve(std::max<size_t>(acc[0] * 12, 16)));
        CUDA_TRY(d_med.reserve(std::max<size_t>(acc[1] * 4, 16)));
        CUDA_TRY(d_frag.reserve(std::max<size_t>(acc[2] * 4, 16)));
        CUDA_TRY(cudaMemcpyAsync(d_off.p, off.data(), (size_t)T * 24, cudaMemcpyHostToDevice, stream_));
        CUDA_TRY(cpmgpu::launch_readout(4, di, K, dp, T, nullptr, (const uint64_t*)d_off.p, (uint32_t*)d_pairs.p,
                                        (uint32_t*)d_med.p, (uint32_t*)d_frag.p, stream_));
        h_pairs.resize(acc[0] * 3);
        h_med.resize(acc[1]);
        h_frag.resize(acc[2]);
        if (acc[0]) CUDA_TRY(cudaMemcpyAsync(h_pairs.data(), d_pairs.p, acc[0] * 12, cudaMemcpyDeviceToHost, stream_));
        if (acc[1]) CUDA_TRY(cudaMemcpyAsync(h_med.data(), d_med.p, acc[1] * 4, cudaMemcpyDeviceToHost, stream_));
        if (acc[2]) CUDA_TRY(cudaMemcpyAsync(h_frag.data(), d_frag.p, acc[2] * 4, cudaMemcpyDeviceToHost, stream_));
        CUDA_TRY(cudaStreamSynchronize(stream_));
        d2h_bytes_ += (size_t)T * 12 + acc[0] * 12 + acc[1] * 4 + acc[2] * 4;
        h2d_bytes_ += (size_t)K * sizeof(ReadoutItem) + (size_t)(K + 1) * 8 + (size_t)T * 24;
        auto split = [&](int k) {
            Topo& t = out[who[k]][s];
            const int64_t ua = prefix[k], ub = prefix[k + 1];
            auto lo = [&](int st) { return off[3 * ua + st]; };
            auto hi = [&](int st) { return ub < T ? off[3 * ub + st] : acc[st]; };
            const size_t np = hi(0) - lo(0);
            t.contact_a.resize(np);
            t.contact_b.resize(np);
            t.contact_n.resize(np);
            for (size_t q = 0; q < np; ++q) {
                const uint32_t* e = &h_pairs[3 * (lo(0) + q)];
                t.contact_a[q] = e[0];
                t.contact_b[q] = e[1];
                t.contact_n[q] = e[2];
            }
            for (uint64_t q = lo(1); q < hi(1); ++q) {
                t.medium_volumes.push_back(h_med[q] & 0x7FFFFFFFu);
                t.medium_touches.push_back((uint8_t)(h_med[q] >> 31));
            }
            t.fragmented.assign(h_frag.begin() + lo(2), h_frag.begin() + hi(2));
        };
        const int nth = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)(K + 63) / 64);
        if (nth <= 1) {
            for (int k = 0; k < K; ++k) split(k);
        } else {
            std::atomic<int> nx{0};
            auto run = [&] { for (int k; (k = nx.fetch_add(1)) < K;) split(k); };
            std::vector<std::thread> th;
            for (int t = 1; t < nth; ++t) th.emplace_back(run);
            run();
            for (auto& t : th) t.join();
        }
    }
    return "";
}

std::string DeviceSims::write_state(size_t i, const std::vector<uint32_t>& padded, const std::vector<uint32_t>& vol,
                                    const std::vector<uint32_t>& itf, const std::vector<int64_t>* sp,
                                    const std::vector<int64_t>* so) {
    const size_t n1 = layouts_[i].n_cells + 1;
    if (padded.size() != (size_t)layouts_[i].g.n_padded || vol.size() != n1 || itf.size() != n1)
        return "write_state: size mismatch";
    // the sweeps index the per-cell arrays by the ids they read from sigma
    for (size_t f = 0; f < padded.size(); ++f)
        if (padded[f] > (uint32_t)layouts_[i].n_cells)
            return "write_state: cell id " + std::to_string(padded[f]) + " at padded index " + std::to_string(f) +
                   " exceeds the number of cells (" + std::to_string(layouts_[i].n_cells) + ")";
    CUDA_TRY(cudaMemcpy(descs_[i].sigma, padded.data(), padded.size() * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(descs_[i].volume, vol.data(), n1 * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(descs_[i].interface, itf.data(), n1 * 4, cudaMemcpyHostToDevice));
    if (sp) CUDA_TRY(cudaMemcpy(descs_[i].sum_pos, sp->data(), sp->size() * 8, cudaMemcpyHostToDevice));
    if (so) CUDA_TRY(cudaMemcpy(descs_[i].sum_outer, so->data(), so->size() * 8, cudaMemcpyHostToDevice));
    return "";
}

// ============================================================ readouts ====
// output.rs:183-231 — closed-form eigenvalues of the symmetric gyration tensor.
static void symmetric_eigenvalues(int D, const double g[3][3], double out[3]) {
    if (D == 2) {
        const double a = g[0][0], b = g[0][1], d = g[1][1];
        const double tr = a + d;
        const double disc = std::sqrt(std::max((a - d) * (a - d) + 4.0 * b * b, 0.0));
        out[0] = (tr + disc) / 2.0;
        out[1] = (tr - disc) / 2.0;
        return;
    }
    const double p1 = g[0][1] * g[0][1] + g[0][2] * g[0][2] + g[1][2] * g[1][2];
    if (p1 == 0.0) { out[0] = g[0][0]; out[1] = g[1][1]; out[2] = g[2][2]; return; }
    const double q = (g[0][0] + g[1][1] + g[2][2]) / 3.0;
    const double a0 = g[0][0] - q, a1 = g[1][1] - q, a2 = g[2][2] - q;
    const double p = std::sqrt((a0 * a0 + a1 * a1 + a2 * a2 + 2.0 * p1) / 6.0);
    auto b = [&](int i, int j) { return (g[i][j] - (i == j ? q : 0.0)) / p; };
    const double det = b(0, 0) * (b(1, 1) * b(2, 2) - b(1, 2) * b(2, 1)) - b(0, 1) * (b(1, 0) * b(2, 2) - b(1, 2) * b(2, 0)) +
                       b(0, 2) * (b(1, 0) * b(2, 1) - b(1, 1) * b(2, 0));
    const double r = std::min(1.0, std::max(-1.0, det / 2.0));
    const double phi = std::acos(r) / 3.0;
    const double e1 = q + 2.0 * p * std::cos(phi);
    const double e3 = q + 2.0 * p * std::cos(phi + 2.0 * M_PI / 3.0);
    out[0] = e1; out[1] = 3.0 * q - e1 - e3; out[2] = e3;
}

// output.rs:147-178 and 289-302
static void cell_summary(int D, uint32_t id, uint32_t vol, uint32_t itf, const int64_t* sp, const int64_t* so,
                         CellSample& o) {
    o.id = id; o.volume = vol; o.interface = itf;
    for (int d = 0; d < 3; ++d) { o.centroid[d] = 0.0; o.eigenvalues[d] = 0.0; }
    const double v = (double)vol;
    for (int d = 0; d < D; ++d) o.centroid[d] = (double)sp[d] / v;
    double g[3][3] = {{0}};
    for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) g[a][b] = (double)so[a * D + b] / v - o.centroid[a] * o.centroid[b];
    double e[3];
    symmetric_eigenvalues(D, g, e);
    for (int i = 1; i < D; ++i)
        for (int j = i; j > 0 && e[j] > e[j - 1]; --j) std::swap(e[j], e[j - 1]);
    double sum = 0.0, sq = 0.0;
    for (int i = 0; i < D; ++i) sum += e[i];
    for (int i = 0; i < D; ++i) sq += e[i] * e[i];
    const double dd = (double)D;
    o.kappa2 = sum > 0.0 ? (dd / (dd - 1.0)) * (sq / (sum * sum)) - 1.0 / (dd - 1.0) : 0.0;
    o.rg2 = sum;
    for (int i = 0; i < D; ++i) o.eigenvalues[i] = e[i];
}

// output.rs:388-420
static bool not_equilibrated(const std::vector<double>& y) {
    const size_t n = y.size();
    if (n < 3) return false;
    double xm = 0.0, ym = 0.0;
    for (size_t i = 0; i < n; ++i) xm += (double)i;
    xm /= (double)n;
    for (size_t i = 0; i < n; ++i) ym += y[i];
    ym /= (double)n;
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < n; ++i) { num += ((double)i - xm) * (y[i] - ym); den += ((double)i - xm) * ((double)i - xm); }
    if (den == 0.0) return false;
    const double slope = num / den, icpt = ym - slope * xm;
    double rv = 0.0;
    for (size_t i = 0; i < n; ++i) { const double r = y[i] - (icpt + slope * (double)i); rv += r * r; }
    const double rs = std::sqrt(rv / (double)n);
    if (rs == 0.0) return std::fabs(slope) * (double)(n - 1) > 0.0;
    return std::fabs(slope) * (double)(n - 1) > 2.0 * rs;
}

// output.rs:456-522 (priority NotEquilibrated > Fragmented > CellLost > Degenerate)
Status run_status(uint32_t min_cell_volume, const std::vector<double>& trace, const std::vector<Sample>& samples,
                  int n_cells, bool have_topology) {
    Status st;
    if (not_equilibrated(trace)) { st.kind = "NotEquilibrated"; return st; }
    if (have_topology)
        for (auto& s : samples)
            if (!s.fragmented.empty()) {
                st.kind = "Fragmented"; st.has_cell = true; st.cell_id = s.fragmented[0]; st.at_mcs = s.mcs;
                return st;
            }
    if (!samples.empty()) {
        size_t window = (size_t)std::ceil((double)samples.size() * 0.5);
        window = std::min(std::max<size_t>(window, 1), samples.size());
        const size_t start = samples.size() - window;
        for (int id = 1; id <= n_cells; ++id) {
            bool all = true;
            for (size_t k = start; k < samples.size(); ++k)
                if (!(samples[k].cells[id - 1].volume <= min_cell_volume)) { all = false; break; }
            if (all) {
                st.kind = "CellLost"; st.has_cell = true; st.cell_id = (uint32_t)id; st.at_mcs = samples[start].mcs;
                return st;
            }
        }
    }
    if (have_topology && n_cells >= 2 && !samples.empty()) {
        const Sample& last = samples.back();
        std::vector<std::vector<uint32_t>> adj(n_cells + 1);
        std::vector<char> present(n_cells + 1, 0);
        uint32_t start = 0;
        for (size_t k = 0; k < last.contact_a.size(); ++k) {
            const uint32_t a = last.contact_a[k], b = last.contact_b[k];
            if (a == 0 || b == 0) continue;
            adj[a].push_back(b); adj[b].push_back(a);
            present[a] = present[b] = 1;
            if (!start) start = a;
        }
        if (start) {
            std::vector<char> vis(n_cells + 1, 0);
            std::vector<uint32_t> stck{start};
            vis[start] = 1;
            size_t cnt = 1;
            while (!stck.empty()) {
                const uint32_t u = stck.back();
                stck.pop_back();
                for (uint32_t w : adj[u]) if (!vis[w]) { vis[w] = 1; ++cnt; stck.push_back(w); }
            }
            if (cnt == (size_t)n_cells) st.kind = "Degenerate";
        }
    }
    return st;
}

static Status status_of(const Config& c, const std::vector<double>& trace, const std::vector<Sample>& samples,
                        int n_cells, bool have_topology) {
    return run_status(c.min_cell_volume, trace, samples, n_cells, have_topology);
}

// Number of energy-trace points the burn-in loop records (output.rs:441-454).
int trace_points(uint64_t burn_in, uint64_t interval, uint64_t start) {
    uint64_t burned = 0;
    int n = 0;
    while (burned < burn_in) {
        burned += std::min(interval, burn_in - burned);
        if (burned >= start) ++n;
    }
    return n;
}

RunPlan plan_for(const Config& c, int sim, bool write_lattice) {
    RunPlan p;
    std::memset(&p, 0, sizeof p);
    p.sim = sim;
    p.burn_in = c.burn_in;
    p.interval = c.interval;
    p.energy_sample_start = c.burn_in - std::min<uint64_t>(c.burn_in, (uint64_t)((double)c.burn_in * 0.25));
    p.n_samples = (int)std::max<uint64_t>(c.readout / std::max<uint64_t>(c.interval, 1), 1);
    p.readout_chunks = (uint64_t)p.n_samples;
    p.write_samples = 1;
    p.write_lattice = write_lattice ? 1 : 0;
    return p;
}

// Reads simulation i of `dev` back after its whole run window and builds
// the run result (output.rs:434-529): samples with per-cell summaries and
// topology readouts, the status, the metadata hashes and the counters.
std::string assemble_result(const Config& c, const Initial& init, const DeviceSims& dev, size_t i, int ns, int nt,
                            const ReadoutOptions& ro, Result& R) {
    const SimLayout& L = dev.layout(i);
    R = Result();
    R.D = c.D;
    for (int d = 0; d < c.D; ++d) R.grid.push_back(c.grid[d]);
    R.used_default = init.used_default;
    for (auto& t : c.types) R.cell_type_names.push_back(t.name);
    R.cell_type_index = init.type_of;
    std::vector<uint32_t> sv, si, slat;
    std::vector<int64_t> ssp, sso;
    std::vector<double> energy;
    std::string e = dev.read_samples(i, ns, sv, si, ssp, sso, ro.include_lattice ? &slat : nullptr);
    if (e.empty()) e = dev.read_energy(i, energy);
    if (e.empty()) e = dev.read_stats(i, R.stats);
    std::vector<uint32_t> fin;
    if (e.empty()) e = dev.read_padded(i, fin);
    if (!e.empty()) return e;
    const int n = L.n_cells, D = c.D;
    const size_t n1 = (size_t)n + 1;
    std::vector<double> trace(energy.begin(), energy.begin() + nt);
    R.samples.resize(ns);
    for (int s = 0; s < ns; ++s) {
        Sample& S = R.samples[s];
        S.mcs = c.burn_in + (uint64_t)(s + 1) * c.interval;
        S.energy = energy[nt + s];
        S.cells.resize(n);
        for (int id = 1; id <= n; ++id)
            cell_summary(D, (uint32_t)id, sv[s * n1 + id], si[s * n1 + id], &ssp[(s * n1 + id) * D],
                         &sso[(s * n1 + id) * D * D], S.cells[id - 1]);
        if (ro.include_lattice) {
            S.lattice.assign(slat.begin() + (size_t)s * L.g.n_sites, slat.begin() + (size_t)(s + 1) * L.g.n_sites);
            S.has_lattice = true;
        }
    }
    if (!ro.topology) R.status = status_of(c, trace, R.samples, n, false);
    R.energy_trace = std::move(trace);
    // metadata (output.rs:66-78): hashes of the final state
    std::vector<uint32_t> fin_int((size_t)L.g.n_sites);
    int64_t x[3] = {0, 0, 0};
    uint64_t occupied = 0;
    for (int64_t q = 0; q < L.g.n_sites; ++q) {
        fin_int[q] = fin[L.g.flat(x)];
        for (int d = D - 1; d >= 0; --d) { if (++x[d] < L.g.dims[d]) break; x[d] = 0; }
    }
    std::vector<uint32_t> vol, itf;
    std::vector<int64_t> sp, so;
    e = dev.read_cells(i, vol, itf, sp, so);
    if (!e.empty()) return e;
    for (size_t id = 1; id < n1; ++id) occupied += vol[id];
    R.metadata.cpm_version = "0.2.0+gb300";
    R.metadata.convention_version = 1;
    R.metadata.convention_hash = convention_hash(c);
    R.metadata.model_hash = model_hash_with(R.metadata.convention_hash, fin_int, init.type_of);
    R.metadata.seed = c.seed;
    R.metadata.seed_policy = "independent";
    R.metadata.derived_phi = (double)(uint32_t)occupied / (double)L.g.n_sites;
    R.metadata.theta_layout_version = 1;
    return "";
}

void attach_topology(const Config& c, std::vector<Topo>& topo, Result& R) {
    for (size_t s = 0; s < R.samples.size() && s < topo.size(); ++s) {
        Sample& S = R.samples[s];
        Topo& t = topo[s];
        S.contact_a = std::move(t.contact_a);
        S.contact_b = std::move(t.contact_b);
        S.contact_n = std::move(t.contact_n);
        S.fragmented = std::move(t.fragmented);
        S.medium_volumes = std::move(t.medium_volumes);
        S.medium_touches = std::move(t.medium_touches);
    }
    R.status = status_of(c, R.energy_trace, R.samples, (int)R.cell_type_index.size(), true);
}

std::string run_many(const std::vector<Config>& configs, const std::vector<Initial>& initials, const ReadoutOptions& ro,
                     std::vector<Result>& out, int device_grid) {
    const size_t N = configs.size();
    out.assign(N, Result());
    if (N == 0) return "";
    const bool snapshots = ro.include_lattice || ro.topology;
    std::vector<RunPlan> plans(N);
    std::vector<int> ns(N), ne(N), nt(N);
    for (size_t i = 0; i < N; ++i) {
        plans[i] = plan_for(configs[i], (int)i, snapshots);
        nt[i] = trace_points(configs[i].burn_in, configs[i].interval, plans[i].energy_sample_start);
        ns[i] = plans[i].n_samples;
        ne[i] = nt[i] + ns[i];
    }
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    // kernels on a non-blocking stream: the read-backs (legacy-stream copies
    // from the assembly threads) then do not wait for them
    cudaStream_t st = nullptr;
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { if (s) cudaStreamDestroy(s); }
    } guard{st};
    DeviceSims dev;
    dev.set_done_tracking(true);
    std::string err = dev.create(configs, initials, ns, ne, snapshots, st);
    if (!err.empty()) return err;
    err = dev.run(plans, device_grid);
    if (!err.empty()) return err;
    const auto t1 = clk::now();
    // ---- assemble results while the device runs: host threads take the
    // simulations in the order the persistent launch serves them (largest
    // first) and start on each as soon as its done flag is set, or once the
    // stream has finished (simulations on other sweeps, or an error, which
    // dev.sync() reports below)
    std::vector<size_t> order(N);
    for (size_t i = 0; i < N; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return dev.layout(a).g.n_sites > dev.layout(b).g.n_sites;
    });
    std::atomic<size_t> next{0};
    std::vector<std::string> errs(N);
    auto worker = [&]() {
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= N) return;
            const size_t i = order[k];
            while (!dev.done(i)) {
                const cudaError_t q = cudaStreamQuery(st);
                if (q != cudaErrorNotReady) break;
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            }
            if (!dev.done(i)) cudaStreamSynchronize(st);
            errs[i] = assemble_result(configs[i], initials[i], dev, i, ns[i], nt[i], ro, out[i]);
        }
    };
    (void)0;
    const unsigned nthreads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)N));
    int dev_id = 0;
    cudaGetDevice(&dev_id);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nthreads; ++t)
        th.emplace_back([&, dev_id] { cudaSetDevice(dev_id); worker(); });
    // topology readouts on the device, queued behind the sweeps
    std::vector<std::vector<Topo>> topo;
    std::string terr;
    if (ro.topology) {
        std::vector<size_t> all(N);
        for (size_t i = 0; i < N; ++i) all[i] = i;
        terr = dev.topology(all, ns, topo);
    }
    cudaStreamSynchronize(st);  // errors are reported by dev.sync() below
    const auto t2 = clk::now();
    for (auto& t : th) t.join();
    err = dev.sync();
    if (!err.empty()) return err;
    if (!terr.empty()) return terr;
    for (auto& e : errs) if (!e.empty()) return e;
    if (ro.topology) {
        std::atomic<size_t> nx{0};
        auto attach = [&]() {
            for (size_t i; (i = nx.fetch_add(1)) < N;) attach_topology(configs[i], topo[i], out[i]);
        };
        std::vector<std::thread> ta;
        for (unsigned t = 1; t < nthreads; ++t) ta.emplace_back(attach);
        attach();
        for (auto& t : ta) t.join();
    }
    const auto t3 = clk::now();
    auto us = [](clk::duration d) { return (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(d).count(); };
    for (auto& R : out) {
        if (R.stats.size() < CPM_STAT_COUNT) R.stats.resize(CPM_STAT_COUNT, 0);
        R.stats[CPM_STAT_H2D_BYTES] = dev.h2d_bytes();
        R.stats[CPM_STAT_D2H_BYTES] = dev.d2h_bytes();
        R.stats[CPM_STAT_HOST_PREP_US] = us(t1 - t0);
        R.stats[CPM_STAT_DEVICE_US] = us(t2 - t1);
        R.stats[CPM_STAT_HOST_READ_US] = us(t3 - t2);
    }
    return "";
}

std::string run_one(const Config& c, const ReadoutOptions& ro, Result& out) {
    std::string e = validate(c);
    if (!e.empty()) return e;
    Initial init;
    e = initialize(c, init);
    if (!e.empty()) return e;
    std::vector<Result> rs;
    e = run_many({c}, {init}, ro, rs);
    if (!e.empty()) return e;
    out = std::move(rs[0]);
    return "";
}

std::string run_batch(const Config& base, const std::vector<std::vector<double>>& thetas, uint64_t master_seed,
                      const ReadoutOptions& ro, std::vector<Result>& out, BatchStage* stage) {
    BatchStage dummy;
    if (!stage) stage = &dummy;
    *stage = BATCH_OK;
    const size_t expected = theta_len(base.types.size());
    for (size_t i = 0; i < thetas.size(); ++i)
        if (thetas[i].size() != expected) {
            *stage = BATCH_THETA;
            return "theta at index " + std::to_string(i) + " has length " + std::to_string(thetas[i].size()) +
                   ", expected " + std::to_string(expected);
        }
    std::vector<Config> cfgs(thetas.size(), base);
    std::vector<Initial> inits(thetas.size());
    std::vector<std::string> errs(thetas.size());
    std::vector<BatchStage> stages(thetas.size(), BATCH_OK);
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= thetas.size()) return;
            std::string e = theta_inject(cfgs[i], thetas[i].data());
            BatchStage at = BATCH_THETA;
            if (e.empty()) { cfgs[i].seed = derive_seed_u64(master_seed, i); e = validate(cfgs[i]); at = BATCH_CONFIG; }
            if (e.empty()) { e = initialize(cfgs[i], inits[i]); at = BATCH_INIT; }
            errs[i] = e;
            if (!e.empty()) stages[i] = at;
        }
    };
    const unsigned nthreads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)std::max<size_t>(thetas.size(), 1)));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nthreads; ++t) th.emplace_back(worker);
    for (auto& t : th) t.join();
    for (size_t i = 0; i < errs.size(); ++i)
        if (!errs[i].empty()) {
            *stage = stages[i];
            return errs[i];
        }
    std::string e = run_many(cfgs, inits, ro, out);
    if (!e.empty()) *stage = BATCH_RUN;
    return e;
}

}  // namespace cpmhost
