// Initial placement of a fresh lattice (host side).
//
// Reproduces the reference's placement bit for bit, including its random
// stream, so a GPU run starts from exactly the lattice the reference would
// start from for the same seed:
//   * explicit placement and its validation (initialization.rs:61-137); the
//     lattice questions (id range, zero volume, connectivity) of a large
//     lattice are answered on the device (cpm_init_device.cu);
//   * default scatter-and-grow (initialization.rs:202-277), drawing from
//     Xoshiro256++ seeded through SplitMix64 (rand_xoshiro 0.6,
//     `seed_from_u64`) with rand 0.8's `gen_range` (widening multiply with
//     the `(range << lz) - 1` acceptance zone): one sequential random
//     stream, so it stays on the host.
// The interface, position sums and gyration accumulator of the placed
// lattice (initialization.rs:396-436) are summed on the device after the
// upload (cpmgpu::launch_derive).
// Growth reads only canonical interior sites, so the halo is not maintained
// here; the device lattice gets its halo when it is padded for upload.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "cpm_host.h"
#include "cpm_kernels.h"

namespace cpmhost {

namespace {
struct Xoshiro256pp {
    uint64_t s[4];
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    explicit Xoshiro256pp(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) {
            x += 0x9e3779b97f4a7c15ULL;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            s[i] = z ^ (z >> 31);
        }
    }
    uint64_t next() {
        const uint64_t r = rotl(s[0] + s[3], 23) + s[0];
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // inclusive [lo, hi]
    uint64_t range_incl(uint64_t lo, uint64_t hi) {
        const uint64_t range = hi - lo + 1;
        if (range == 0) return next();
        const uint64_t zone = (range << __builtin_clzll(range)) - 1;
        for (;;) {
            const unsigned __int128 m = (unsigned __int128)next() * range;
            if ((uint64_t)m <= zone) return lo + (uint64_t)(m >> 64);
        }
    }
    uint64_t range(uint64_t lo, uint64_t hi_excl) { return range_incl(lo, hi_excl - 1); }
};
}  // namespace

void Geometry::init(const Config& c) {
    D = c.D;
    periodic = c.periodic;
    for (int d = 0; d < 3; ++d) { dims[d] = d < D ? c.grid[d] : 1; pdims[d] = d < D ? c.grid[d] + 2 : 1; }
    int64_t s = 1;
    for (int d = D - 1; d >= 0; --d) { strides[d] = s; s *= pdims[d]; }
    for (int d = D; d < 3; ++d) strides[d] = 0;
    n_padded = s;
    n_sites = 1;
    for (int d = 0; d < D; ++d) n_sites *= dims[d];
}

int64_t Geometry::flat(const int64_t* x) const {
    int64_t f = 0;
    for (int d = 0; d < D; ++d) f += (x[d] + 1) * strides[d];
    return f;
}

// Interior copy plus the halo: medium for a fixed boundary, the mirrored
// opposite face for a periodic one (lattice.rs:199-254).
std::vector<uint32_t> pad_lattice(const Geometry& g, const std::vector<uint32_t>& in) {
    std::vector<uint32_t> p((size_t)g.n_padded, 0);
    int64_t pc[3] = {0, 0, 0};
    for (int64_t f = 0; f < g.n_padded; ++f) {
        int64_t r = f;
        bool halo = false;
        int64_t ic[3] = {0, 0, 0};
        for (int d = 0; d < g.D; ++d) {
            pc[d] = r / g.strides[d];
            r %= g.strides[d];
            if (pc[d] == 0 || pc[d] == g.pdims[d] - 1) halo = true;
            ic[d] = pc[d] == 0 ? g.dims[d] - 1 : (pc[d] == g.pdims[d] - 1 ? 0 : pc[d] - 1);
        }
        if (halo && !g.periodic) continue;
        int64_t q = 0;
        for (int d = 0; d < g.D; ++d) q = q * g.dims[d] + ic[d];
        p[f] = in[q];
    }
    return p;
}

namespace {
struct Placer {
    const Config& c;
    Geometry g;
    std::vector<uint32_t> lat;  // padded; only interior entries are meaningful
    std::vector<int64_t> copy_off;
    // canon[f]: f for an interior site; for a halo site its periodic image
    // (periodic) or -1 (fixed: not a site). One lookup replaces the per-axis
    // divisions of `interior` / `wrapped` on the growth path.
    std::vector<int32_t> canon;
    explicit Placer(const Config& cfg) : c(cfg) {
        g.init(cfg);
        lat.assign((size_t)g.n_padded, 0);
        for (auto& o : stencil(NBH_VON_NEUMANN, cfg.D)) {
            int64_t d = 0;
            for (int a = 0; a < cfg.D; ++a) d += o[a] * g.strides[a];
            copy_off.push_back(d);
        }
        canon.resize((size_t)g.n_padded);
        int64_t pc[3] = {0, 0, 0};
        for (int64_t f = 0; f < g.n_padded; ++f) {
            bool halo = false;
            int64_t ic[3] = {0, 0, 0};
            for (int d = 0; d < g.D; ++d) {
                if (pc[d] == 0 || pc[d] == g.pdims[d] - 1) halo = true;
                ic[d] = pc[d] == 0 ? g.dims[d] - 1 : (pc[d] == g.pdims[d] - 1 ? 0 : pc[d] - 1);
            }
            canon[f] = !halo ? (int32_t)f : (g.periodic ? (int32_t)g.flat(ic) : -1);
            for (int d = g.D - 1; d >= 0; --d) { if (++pc[d] < g.pdims[d]) break; pc[d] = 0; }
        }
    }
    // initialization.rs:173-187 / 303-318
    int64_t canonical(int64_t f, int64_t off) const {
        const int64_t nb = f + off;
        return g.periodic ? canon[nb] : nb;
    }
    bool growable(int64_t f, int64_t off, int64_t& out) const {
        const int32_t c2 = canon[f + off];
        if (c2 < 0) return false;
        out = c2;
        return true;
    }
    double distance(const int64_t* a, const int64_t* b) const {
        double s = 0.0;
        for (int d = 0; d < g.D; ++d) {
            const double raw = std::fabs((double)a[d] - (double)b[d]);
            const double delta = g.periodic ? std::min(raw, (double)g.dims[d] - raw) : raw;
            s += delta * delta;
        }
        return std::sqrt(s);
    }
    // Size of the connected component (connectivity is von Neumann) holding
    // each cell's first site in scan order, for all cells in one pass over
    // the lattice; a cell is connected when that size equals its volume.
    std::vector<uint64_t> first_component_sizes(size_t n) const {
        std::vector<int64_t> first(n + 1, -1);
        int64_t x[3] = {0, 0, 0};
        for (int64_t i = 0; i < g.n_sites; ++i) {
            const int64_t f = g.flat(x);
            const uint32_t id = lat[f];
            if (id && id <= n && first[id] < 0) first[id] = f;
            for (int d = g.D - 1; d >= 0; --d) { if (++x[d] < g.dims[d]) break; x[d] = 0; }
        }
        std::vector<uint64_t> size(n + 1, 0);
        std::vector<char> vis(lat.size(), 0);
        std::vector<int64_t> st;
        for (size_t id = 1; id <= n; ++id) {
            if (first[id] < 0) continue;
            st.assign(1, first[id]);
            vis[first[id]] = 1;
            uint64_t c = 1;
            while (!st.empty()) {
                const int64_t f = st.back();
                st.pop_back();
                for (int64_t off : copy_off) {
                    const int64_t nb = canonical(f, off);
                    if (lat[nb] == id && !vis[nb]) { vis[nb] = 1; ++c; st.push_back(nb); }
                }
            }
            size[id] = c;
        }
        return size;
    }
    std::vector<uint32_t> interior_copy() const {
        std::vector<uint32_t> out((size_t)g.n_sites);
        int64_t x[3] = {0, 0, 0};
        for (int64_t i = 0; i < g.n_sites; ++i) {
            out[i] = lat[g.flat(x)];
            for (int d = g.D - 1; d >= 0; --d) { if (++x[d] < g.dims[d]) break; x[d] = 0; }
        }
        return out;
    }
};
}  // namespace

// Explicit lattices of at least this many sites are checked on the device
// when the process has one (CPM_GPU_INIT_DEVICE_MIN_SITES overrides the
// default of 65,536; "0" sends every explicit lattice there); smaller ones,
// and every lattice in a process without a GPU, here. Both give the same
// verdict and message.
static int64_t device_check_min_sites() {
    static const bool has_device = [] {
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
            cudaGetLastError();
            return false;
        }
        return true;
    }();
    if (!has_device) return INT64_MAX;
    const char* e = std::getenv("CPM_GPU_INIT_DEVICE_MIN_SITES");
    return e ? (int64_t)std::strtoll(e, nullptr, 10) : (int64_t)65536;
}

std::string initialize(const Config& c, Initial& out) {
    const int64_t ns = n_sites(c);
    const int ntypes = (int)c.types.size();
    if (c.init_explicit) {
        out.used_default = false;
        if ((int64_t)c.init_lattice.size() != ns)
            return "explicit lattice has " + std::to_string(c.init_lattice.size()) + " entries, expected N_sites = " +
                   std::to_string(ns);
        const size_t n = c.init_type_of.size();
        for (size_t i = 0; i < n; ++i)
            if (c.init_type_of[i] >= (uint64_t)ntypes)
                return "cell " + std::to_string(i + 1) + " has type_index " + std::to_string(c.init_type_of[i]) +
                       ", but only " + std::to_string(ntypes) + " types are declared";
        // the placement, once every check has passed
        auto accept = [&]() -> std::string {
            out.lattice = c.init_lattice;
            out.type_of.assign(n, 0);
            for (size_t i = 0; i < n; ++i) out.type_of[i] = (uint32_t)c.init_type_of[i];
            return "";
        };
        const std::string not_connected =
            " is not connected under connectivity_neighborhood — every explicitly-placed cell must already be connected";
        if (ns >= device_check_min_sites() && n < 0xFFFFFFFFull) {
            // the lattice questions on the device: one upload, a union-find
            cpmgpu::ExplicitCheck ck;
            const cudaError_t ce = cpmgpu::check_explicit_lattice(c.D, c.grid, c.periodic ? 1 : 0, c.init_lattice.data(),
                                                                  ns, (uint32_t)n, &ck);
            if (ce != cudaSuccess) return std::string("CUDA error: ") + cudaGetErrorString(ce);
            if (ck.first_bad_site >= 0)
                return "lattice references cell id " + std::to_string(c.init_lattice[ck.first_bad_site]) +
                       ", but cell_type_of only covers " + std::to_string(n) + " cells";
            if (ck.zero_volume_id) return "cell " + std::to_string(ck.zero_volume_id) + " has zero volume in the supplied lattice";
            if (ck.disconnected_id) return "cell " + std::to_string(ck.disconnected_id) + not_connected;
            return accept();
        }
        for (uint32_t id : c.init_lattice)
            if ((size_t)id > n)
                return "lattice references cell id " + std::to_string(id) + ", but cell_type_of only covers " +
                       std::to_string(n) + " cells";
        Placer P(c);
        std::vector<uint32_t> vol(n, 0);
        int64_t x[3] = {0, 0, 0};
        for (int64_t i = 0; i < ns; ++i) {
            const uint32_t v = c.init_lattice[i];
            P.lat[P.g.flat(x)] = v;
            if (v) vol[v - 1] += 1;
            for (int d = P.g.D - 1; d >= 0; --d) { if (++x[d] < P.g.dims[d]) break; x[d] = 0; }
        }
        for (size_t i = 0; i < n; ++i)
            if (vol[i] == 0) return "cell " + std::to_string(i + 1) + " has zero volume in the supplied lattice";
        const std::vector<uint64_t> comp = P.first_component_sizes(n);
        for (size_t id = 1; id <= n; ++id)
            if (comp[id] != vol[id - 1]) return "cell " + std::to_string(id) + not_connected;
        return accept();
    }
    // ---- scatter and grow ----
    Placer P(c);
    out.used_default = true;
    std::vector<uint32_t> tcell;
    for (size_t t = 0; t < c.cell_counts.size(); ++t)
        for (uint64_t k = 0; k < c.cell_counts[t]; ++k) tcell.push_back((uint32_t)t);
    const int n = (int)tcell.size();
    if (n == 0) return "cell_counts sums to zero cells — nothing to place";
    double avg = 0.0;
    for (auto& t : c.types) avg += (double)t.target_volume;
    avg /= (double)c.types.size();
    const double min_sep = std::sqrt(avg / M_PI);
    Xoshiro256pp rng(c.seed);
    std::vector<std::array<int64_t, 3>> seeds;
    seeds.reserve(n);
    // Seeds in buckets at least min_sep wide per axis: a seed closer than
    // min_sep to a candidate lies in the candidate's bucket or a neighbouring
    // one (wrapping on periodic axes), so only those are compared. The
    // verdict and the draws are those of comparing against every seed.
    int nbk[3] = {1, 1, 1};
    bool bucketed = true;
    for (int d = 0; d < c.D; ++d) {
        nbk[d] = std::max<int64_t>(1, (int64_t)std::floor((double)P.g.dims[d] / std::max(min_sep, 1e-9)));
        if (nbk[d] < 3) bucketed = false;
    }
    std::vector<std::vector<int>> buckets(bucketed ? (size_t)nbk[0] * nbk[1] * nbk[2] : 0);
    auto bucket_of = [&](const int64_t* x, int* b) {
        for (int d = 0; d < 3; ++d) b[d] = d < c.D ? (int)(x[d] * nbk[d] / P.g.dims[d]) : 0;
    };
    auto too_close = [&](const std::array<int64_t, 3>& cand) {
        if (!bucketed) {
            for (auto& q : seeds)
                if (!(P.distance(q.data(), cand.data()) >= min_sep)) return true;
            return false;
        }
        int b[3];
        bucket_of(cand.data(), b);
        for (int dz = c.D > 2 ? -1 : 0; dz <= (c.D > 2 ? 1 : 0); ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    int q[3] = {b[0] + dx, b[1] + dy, b[2] + dz};
                    bool skip = false;
                    for (int d = 0; d < c.D; ++d) {
                        if (q[d] < 0 || q[d] >= nbk[d]) {
                            if (!P.g.periodic) { skip = true; break; }
                            q[d] = (q[d] + nbk[d]) % nbk[d];
                        }
                    }
                    if (skip) continue;
                    for (int k : buckets[((size_t)q[0] * nbk[1] + q[1]) * nbk[2] + q[2]])
                        if (!(P.distance(seeds[k].data(), cand.data()) >= min_sep)) return true;
                }
        return false;
    };
    for (int s = 0; s < n; ++s) {
        bool placed = false;
        for (int a = 0; a < 20000; ++a) {
            std::array<int64_t, 3> cand{0, 0, 0};
            for (int d = 0; d < c.D; ++d) cand[d] = (int64_t)rng.range(0, (uint64_t)P.g.dims[d]);
            if (!too_close(cand)) {
                seeds.push_back(cand);
                if (bucketed) {
                    int b[3];
                    bucket_of(cand.data(), b);
                    buckets[((size_t)b[0] * nbk[1] + b[1]) * nbk[2] + b[2]].push_back((int)seeds.size() - 1);
                }
                placed = true;
                break;
            }
        }
        if (!placed) {
            char buf[64];
            std::snprintf(buf, sizeof buf, "%.2f", min_sep);
            std::string grid = "[";
            for (int d = 0; d < c.D; ++d) { if (d) grid += ", "; grid += std::to_string(c.grid[d]); }
            grid += "]";
            return "could not place all " + std::to_string(n) + " seed points with minimum separation " + buf +
                   " on a grid of " + grid + " — too crowded for this configuration";
        }
    }
    std::vector<uint32_t> vol(n, 0);
    for (int i = 0; i < n; ++i) { P.lat[P.g.flat(seeds[i].data())] = (uint32_t)(i + 1); vol[i] = 1; }
    std::vector<uint32_t> target(n);
    for (int i = 0; i < n; ++i) target[i] = c.types[tcell[i]].target_volume;
    std::vector<std::vector<int64_t>> frontier(n);
    for (int i = 0; i < n; ++i) {
        const int64_t sf = P.g.flat(seeds[i].data());
        for (int64_t off : P.copy_off) {
            int64_t nb;
            if (P.growable(sf, off, nb) && P.lat[nb] == 0) frontier[i].push_back(nb);
        }
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    for (;;) {
        bool grew = false;
        for (int oi = 0; oi < n; ++oi) {
            const int i = order[oi];
            if (vol[i] >= target[i]) continue;
            auto& fr = frontier[i];
            fr.erase(std::remove_if(fr.begin(), fr.end(), [&](int64_t f) { return P.lat[f] != 0; }), fr.end());
            if (fr.empty()) continue;
            const size_t pick = (size_t)rng.range(0, fr.size());
            const int64_t claimed = fr[pick];
            fr[pick] = fr.back();
            fr.pop_back();
            P.lat[claimed] = (uint32_t)(i + 1);
            vol[i] += 1;
            for (int64_t off : P.copy_off) {
                int64_t nb;
                if (P.growable(claimed, off, nb) && P.lat[nb] == 0) fr.push_back(nb);
            }
            grew = true;
        }
        if (!grew) break;
        for (int i = n - 1; i >= 1; --i) {
            const int j = (int)rng.range_incl(0, (uint64_t)i);
            std::swap(order[i], order[j]);
        }
    }
    out.lattice = P.interior_copy();
    out.type_of = tcell;
    return "";
}

// ----------------------------------------------------------- simple points --
// Adjacency bitmasks of the canonical full shell (simple_point.rs:197-213):
// face = Manhattan distance 1, full = Chebyshev distance 1.
void simple_point_masks(int D, uint32_t* face_adj, uint32_t* full_adj, uint32_t* origin_face_mask) {
    std::vector<std::array<int, 3>> offs = stencil(D == 2 ? NBH_MOORE : NBH_TWENTY_SIX, D);
    const int n = (int)offs.size();
    *origin_face_mask = 0;
    for (int i = 0; i < n; ++i) {
        face_adj[i] = full_adj[i] = 0;
        int mo = 0;
        for (int d = 0; d < D; ++d) mo += std::abs(offs[i][d]);
        if (mo == 1) *origin_face_mask |= 1u << i;
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            int m = 0, cheb = 0;
            for (int d = 0; d < D; ++d) { const int a = std::abs(offs[i][d] - offs[j][d]); m += a; cheb = std::max(cheb, a); }
            if (m == 1) face_adj[i] |= 1u << j;
            if (cheb <= 1) full_adj[i] |= 1u << j;
        }
    }
}

static uint32_t flood(uint32_t comp, uint32_t universe, const uint32_t* adj, int n) {
    for (;;) {
        uint32_t before = comp;
        for (int i = 0; i < n; ++i)
            if ((comp >> i) & 1u) comp |= adj[i] & universe;
        if (comp == before) return comp;
    }
}

// simple_point.rs:242-306: simple iff the complement is one component under
// full adjacency and exactly one face-component of the object touches x.
void table2d(uint32_t out[8]) {
    uint32_t face[26], full[26], origin;
    simple_point_masks(2, face, full, &origin);
    for (int w = 0; w < 8; ++w) out[w] = 0;
    for (uint32_t obj = 0; obj < 256; ++obj) {
        const uint32_t cm = (~obj) & 0xFFu;
        int comps = 0;
        for (uint32_t rem = cm; rem;) { rem &= ~flood(1u << __builtin_ctz(rem), cm, full, 8); ++comps; }
        if (comps != 1) continue;
        int touching = 0;
        for (uint32_t rem = obj; rem;) {
            const uint32_t cc = flood(1u << __builtin_ctz(rem), obj, face, 8);
            rem &= ~cc;
            if (cc & origin) ++touching;
        }
        if (touching == 1) out[obj >> 5] |= 1u << (obj & 31);
    }
}

}  // namespace cpmhost
