// CPU restatement of the DebajyotiS/cpm-rust `cpm-core` hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the correctness oracle for the
// GB300 engine: it is imported by `tests/`, by `__graft_entry__.smoke()` to
// compare one small device run against, and by `bench.py` for the timed CPU
// baseline (and the `--impl reference` arm). The product path never links or
// calls it.
//
// Parity status: pinned. The restatement reproduces the reference's frozen
// 2D trajectory bit for bit (crates/cpm-core/tests/dimension_consistency.rs:
// 113-131: V=[7,9], I=[28,32], energy bits 4638468362461406824, model_hash
// 60ec713d...) and the published derived seeds for master_seed=42
// (notebooks/batch_execution_demo.ipynb, cell 7), and the calibrated target
// interfaces 74.753 / 66.097 to all printed decimals (tests/calibration.rs,
// config.rs:588-595: one cell on a 60x60 fixed lattice, 40,000 MCS, a second
// frozen trajectory). `tests/test_oracle_kat.py` checks them. The loop's
// other modes (Metropolis-Hastings acceptance, monte_carlo.rs:168-224; the
// Act term, energy.rs:329-471) have no frozen trajectory in the reference;
// the Act term is pinned against the scenarios of the reference's own unit
// tests (energy.rs:955-1300), the MH decision against its formula
// (`tests/test_oracle_modes.py`), and the MH chain against the exact
// Boltzmann distribution of the reference's harness
// (tests/exact_boltzmann.rs; `tests/test_oracle_boltzmann.py`).
//
// Every function cites the reference file:line it restates. The third-party
// arithmetic the reference pulls from crates that are not vendored in the
// reference tree is restated from the published algorithms:
//   * rand_xoshiro 0.6.0: Xoshiro256++ (Blackman & Vigna) seeded through
//     SplitMix64 (`seed_from_u64`), 64-bit output.
//   * rand 0.8.x: `gen_range` on usize = widening-multiply rejection with
//     the "zone = (range << lz(range)) - 1" acceptance test, and `gen::<f64>`
//     = (next_u64 >> 11) * 2^-53.
//   * blake3 1.8.7: the BLAKE3 hash (O'Connor et al., BLAKE3 specification):
//     7-round compression, 1024-byte chunks, binary merkle tree.
//   * serde_json: compact JSON with fields in declaration order, used for the
//     convention and model hashes (crates/cpm-core/src/config.rs:423-556).
//   * libm exp and pow: the reference calls f64::exp / f64::powf (glibc on
//     Linux); so do we.
//
// Build: see oracle/Makefile (gcc -O2 -ffp-contract=off; Rust never fuses
// multiply-add, so neither may we).

#include <cstdint>
#include <cstring>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>
#include <deque>
#include <algorithm>
#include <thread>
#include <atomic>
#include <map>
#include <memory>
#include <array>

namespace orc {

// ===========================================================================
// RNG: rand_xoshiro 0.6 Xoshiro256++ + rand 0.8 sampling.
// Call sites: crates/cpm-core/src/rng.rs:12-14 (seed_from_u64),
// monte_carlo.rs:39,57,158 and initialization.rs:235,290,313 (sampling).
// ===========================================================================
static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Xoshiro {
    uint64_t s[4];
    uint64_t next_u64() {
        const uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl64(s[3], 45);
        return result;
    }
};

static inline uint64_t splitmix_next(uint64_t& x) {
    x += 0x9e3779b97f4a7c15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// rng.rs:12-14 -> Xoshiro256PlusPlus::seed_from_u64: the 32-byte seed is four
// SplitMix64 outputs (little-endian), so state word i is output i.
static Xoshiro xoshiro_from_u64(uint64_t seed) {
    Xoshiro r;
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) r.s[i] = splitmix_next(x);
    if ((r.s[0] | r.s[1] | r.s[2] | r.s[3]) == 0) return xoshiro_from_u64(0);
    return r;
}

// rand 0.8 UniformInt<usize>::sample_single_inclusive on a 64-bit target.
static uint64_t gen_range_incl(Xoshiro& rng, uint64_t low, uint64_t high) {
    const uint64_t range = high - low + 1;
    if (range == 0) return rng.next_u64();
    const int lz = __builtin_clzll(range);
    const uint64_t zone = (range << lz) - 1;
    for (;;) {
        const uint64_t v = rng.next_u64();
        const unsigned __int128 m = (unsigned __int128)v * (unsigned __int128)range;
        const uint64_t hi = (uint64_t)(m >> 64);
        const uint64_t lo = (uint64_t)m;
        if (lo <= zone) return low + hi;
    }
}
// `gen_range(low..high)` = sample_single_inclusive(low, high - 1).
static inline uint64_t gen_range(Xoshiro& rng, uint64_t low, uint64_t high) {
    return gen_range_incl(rng, low, high - 1);
}
// rand 0.8 Standard for f64: 53 high bits times 2^-53.
static inline double gen_f64(Xoshiro& rng) {
    const uint64_t v = rng.next_u64() >> 11;
    return (1.0 / 9007199254740992.0) * (double)v;
}

// ===========================================================================
// BLAKE3 (published specification), used by rng.rs:20-40 and
// config.rs:511,555.
// ===========================================================================
namespace b3 {
static const uint32_t IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                               0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
static const int PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
enum { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };
static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
static inline void g(uint32_t* v, int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] = v[a] + v[b] + x; v[d] = rotr(v[d] ^ v[a], 16);
    v[c] = v[c] + v[d];     v[b] = rotr(v[b] ^ v[c], 12);
    v[a] = v[a] + v[b] + y; v[d] = rotr(v[d] ^ v[a], 8);
    v[c] = v[c] + v[d];     v[b] = rotr(v[b] ^ v[c], 7);
}
static void compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                     uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t v[16];
    for (int i = 0; i < 8; ++i) v[i] = cv[i];
    for (int i = 0; i < 4; ++i) v[8 + i] = IV[i];
    v[12] = (uint32_t)counter; v[13] = (uint32_t)(counter >> 32);
    v[14] = block_len; v[15] = flags;
    uint32_t m[16];
    for (int i = 0; i < 16; ++i) m[i] = block[i];
    for (int r = 0; r < 7; ++r) {
        g(v, 0, 4, 8, 12, m[0], m[1]);   g(v, 1, 5, 9, 13, m[2], m[3]);
        g(v, 2, 6, 10, 14, m[4], m[5]);  g(v, 3, 7, 11, 15, m[6], m[7]);
        g(v, 0, 5, 10, 15, m[8], m[9]);  g(v, 1, 6, 11, 12, m[10], m[11]);
        g(v, 2, 7, 8, 13, m[12], m[13]); g(v, 3, 4, 9, 14, m[14], m[15]);
        if (r < 6) {
            uint32_t t[16];
            for (int i = 0; i < 16; ++i) t[i] = m[PERM[i]];
            for (int i = 0; i < 16; ++i) m[i] = t[i];
        }
    }
    for (int i = 0; i < 8; ++i) { out[i] = v[i] ^ v[i + 8]; out[i + 8] = v[i + 8] ^ cv[i]; }
}
static void load_block(const uint8_t* p, size_t n, uint32_t w[16]) {
    uint8_t buf[64];
    std::memset(buf, 0, 64);
    std::memcpy(buf, p, n);
    for (int i = 0; i < 16; ++i)
        w[i] = (uint32_t)buf[4 * i] | ((uint32_t)buf[4 * i + 1] << 8) |
               ((uint32_t)buf[4 * i + 2] << 16) | ((uint32_t)buf[4 * i + 3] << 24);
}
// Chaining value of one chunk; `root` set only when the whole input is one chunk.
static void chunk_cv(const uint8_t* p, size_t n, uint64_t chunk_index, bool root, uint32_t out[8]) {
    uint32_t cv[8];
    for (int i = 0; i < 8; ++i) cv[i] = IV[i];
    const size_t nblocks = n == 0 ? 1 : (n + 63) / 64;
    for (size_t b = 0; b < nblocks; ++b) {
        const size_t off = b * 64;
        const size_t len = std::min<size_t>(64, n - std::min(n, off));
        uint32_t w[16];
        load_block(p + off, len, w);
        uint32_t flags = 0;
        if (b == 0) flags |= CHUNK_START;
        if (b == nblocks - 1) { flags |= CHUNK_END; if (root) flags |= ROOT; }
        uint32_t o[16];
        compress(cv, w, chunk_index, (uint32_t)len, flags, o);
        for (int i = 0; i < 8; ++i) cv[i] = o[i];
    }
    for (int i = 0; i < 8; ++i) out[i] = cv[i];
}
static void parent_cv(const uint32_t l[8], const uint32_t r[8], bool root, uint32_t out[8]) {
    uint32_t w[16];
    for (int i = 0; i < 8; ++i) { w[i] = l[i]; w[8 + i] = r[i]; }
    uint32_t o[16];
    compress(IV, w, 0, 64, PARENT | (root ? ROOT : 0), o);
    for (int i = 0; i < 8; ++i) out[i] = o[i];
}
// Tree hash over chunks [first, first+count): the left subtree holds the
// largest power-of-two number of chunks strictly less than `count`.
static void subtree(const uint8_t* data, size_t len, uint64_t first, uint64_t count, bool root, uint32_t out[8]) {
    if (count == 1) {
        const size_t off = (size_t)first * 1024;
        chunk_cv(data + off, std::min<size_t>(1024, len - off), first, root, out);
        return;
    }
    uint64_t left = 1;
    while (left * 2 < count) left *= 2;
    uint32_t l[8], r[8];
    subtree(data, len, first, left, false, l);
    subtree(data, len, first + left, count - left, false, r);
    parent_cv(l, r, root, out);
}
static void hash(const uint8_t* data, size_t len, uint8_t out[32]) {
    const uint64_t nchunks = len == 0 ? 1 : (len + 1023) / 1024;
    uint32_t h[8];
    subtree(data, len, 0, nchunks, true, h);
    for (int i = 0; i < 8; ++i)
        for (int b = 0; b < 4; ++b) out[4 * i + b] = (uint8_t)(h[i] >> (8 * b));
}
static std::string hex(const uint8_t d[32]) {
    static const char* digits = "0123456789abcdef";
    std::string s;
    for (int i = 0; i < 32; ++i) { s += digits[d[i] >> 4]; s += digits[d[i] & 15]; }
    return s;
}
}  // namespace b3

// rng.rs:20-40: first 8 little-endian bytes of BLAKE3(master LE || index LE).
static uint64_t derive_seed_u64(uint64_t master, uint64_t index) {
    uint8_t in[16];
    for (int i = 0; i < 8; ++i) { in[i] = (uint8_t)(master >> (8 * i)); in[8 + i] = (uint8_t)(index >> (8 * i)); }
    uint8_t out[32];
    b3::hash(in, 16, out);
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)out[i] << (8 * i);
    return v;
}

// ===========================================================================
// Stencils: neighborhood.rs:45-137. Offset ORDER is part of the RNG contract.
// ===========================================================================
enum NbhKind { NBH_VON_NEUMANN = 0, NBH_MOORE = 1, NBH_EIGHTEEN = 2, NBH_TWENTY_SIX = 3, NBH_TWENTY_SIX_WEIGHTED = 4 };

struct Off { int c[3]; };

// neighborhood.rs:45-56: [+e0, -e0, +e1, -e1, (+e2, -e2)].
static std::vector<Off> von_neumann(int D) {
    std::vector<Off> v;
    for (int a = 0; a < D; ++a) {
        Off p{{0, 0, 0}}, m{{0, 0, 0}};
        p.c[a] = 1; m.c[a] = -1;
        v.push_back(p); v.push_back(m);
    }
    return v;
}
// neighborhood.rs:75-95: base-3 code, digit for axis 0 varies fastest.
static std::vector<Off> full_moore(int D) {
    int total = 1;
    for (int d = 0; d < D; ++d) total *= 3;
    std::vector<Off> v;
    for (int code = 0; code < total; ++code) {
        int c = code, nz = 0;
        Off o{{0, 0, 0}};
        for (int d = 0; d < D; ++d) { o.c[d] = (c % 3) - 1; c /= 3; if (o.c[d]) ++nz; }
        if (nz > 0) v.push_back(o);
    }
    return v;
}
// neighborhood.rs:109-115: full shell filtered to <= 2 nonzero components.
static std::vector<Off> eighteen() {
    std::vector<Off> v;
    for (const Off& o : full_moore(3)) {
        int nz = (o.c[0] != 0) + (o.c[1] != 0) + (o.c[2] != 0);
        if (nz <= 2) v.push_back(o);
    }
    return v;
}
static bool stencil_for(int kind, int D, std::vector<Off>& out) {
    switch (kind) {
        case NBH_VON_NEUMANN: out = von_neumann(D); return true;
        case NBH_MOORE: if (D != 2) return false; out = full_moore(2); return true;
        case NBH_EIGHTEEN: if (D != 3) return false; out = eighteen(); return true;
        case NBH_TWENTY_SIX: if (D != 3) return false; out = full_moore(3); return true;
        default: return false;  // weighted stencils are rejected by validation
    }
}

// ===========================================================================
// Simple points: simple_point.rs:38-366 (FastChecker bitmask flood fill).
// ===========================================================================
struct FastChecker {
    int n = 0;
    uint32_t face_adj[26], full_adj[26];
    uint32_t origin_face_mask = 0, full_mask = 0;
    void init(int D) {
        std::vector<Off> offs = full_moore(D);
        n = (int)offs.size();
        auto face = [&](const Off& a, const Off& b) {
            int m = 0;
            for (int d = 0; d < D; ++d) m += std::abs(a.c[d] - b.c[d]);
            return m == 1;
        };
        auto full = [&](const Off& a, const Off& b) {
            bool same = true, close = true;
            for (int d = 0; d < D; ++d) { if (a.c[d] != b.c[d]) same = false; if (std::abs(a.c[d] - b.c[d]) > 1) close = false; }
            return !same && close;
        };
        Off origin{{0, 0, 0}};
        origin_face_mask = 0;
        for (int i = 0; i < n; ++i) {
            face_adj[i] = full_adj[i] = 0;
            for (int j = 0; j < n; ++j) {
                if (i == j) continue;
                if (face(offs[i], offs[j])) face_adj[i] |= 1u << j;
                if (full(offs[i], offs[j])) full_adj[i] |= 1u << j;
            }
            if (face(offs[i], origin)) origin_face_mask |= 1u << i;
        }
        full_mask = (uint32_t)((1ULL << n) - 1);
    }
    uint32_t flood(uint32_t comp, uint32_t universe, const uint32_t* adj) const {
        for (;;) {
            uint32_t before = comp;
            for (int i = 0; i < n; ++i)
                if ((comp >> i) & 1u) comp |= adj[i] & universe;
            if (comp == before) return comp;
        }
    }
    bool is_simple(uint32_t object) const {
        uint32_t comp_mask = (~object) & full_mask;
        int count = 0;
        uint32_t rem = comp_mask;
        while (rem) {
            int s = __builtin_ctz(rem);
            rem &= ~flood(1u << s, comp_mask, full_adj);
            ++count;
        }
        if (count != 1) return false;
        int touching = 0;
        rem = object;
        while (rem) {
            int s = __builtin_ctz(rem);
            uint32_t c = flood(1u << s, object, face_adj);
            rem &= ~c;
            if (c & origin_face_mask) ++touching;
        }
        return touching == 1;
    }
};
// Built once per process on first use; function-local statics initialise
// thread-safely, so simulations on several host threads may race to it.
static FastChecker& checker(int D) {
    if (D == 2) {
        static FastChecker c2 = [] { FastChecker c; c.init(2); return c; }();
        return c2;
    }
    static FastChecker c3 = [] { FastChecker c; c.init(3); return c; }();
    return c3;
}

// Slow reference checker (simple_point.rs:52-117): explicit component lists.
static bool slow_is_simple(int D, uint32_t object) {
    std::vector<Off> offs = full_moore(D);
    const int n = (int)offs.size();
    auto face = [&](const Off& a, const Off& b) { int m = 0; for (int d = 0; d < D; ++d) m += std::abs(a.c[d] - b.c[d]); return m == 1; };
    auto full = [&](const Off& a, const Off& b) {
        bool same = true, close = true;
        for (int d = 0; d < D; ++d) { if (a.c[d] != b.c[d]) same = false; if (std::abs(a.c[d] - b.c[d]) > 1) close = false; }
        return !same && close;
    };
    auto comps = [&](const std::vector<bool>& mask, bool use_face) {
        std::vector<std::vector<int>> out;
        std::vector<bool> vis(n, false);
        for (int s = 0; s < n; ++s) {
            if (!mask[s] || vis[s]) continue;
            vis[s] = true;
            std::vector<int> st{s}, comp{s};
            while (!st.empty()) {
                int i = st.back(); st.pop_back();
                for (int j = 0; j < n; ++j)
                    if (mask[j] && !vis[j] && (use_face ? face(offs[i], offs[j]) : full(offs[i], offs[j]))) {
                        vis[j] = true; st.push_back(j); comp.push_back(j);
                    }
            }
            out.push_back(comp);
        }
        return out;
    };
    std::vector<bool> obj(n), cmp(n);
    for (int i = 0; i < n; ++i) { obj[i] = (object >> i) & 1u; cmp[i] = !obj[i]; }
    if (comps(cmp, false).size() != 1) return false;
    Off origin{{0, 0, 0}};
    int touching = 0;
    for (auto& c : comps(obj, true)) {
        bool t = false;
        for (int i : c) if (face(offs[i], origin)) t = true;
        if (t) ++touching;
    }
    return touching == 1;
}

// ===========================================================================
// Configuration (config.rs:262-282, cell.rs:13-26).
// ===========================================================================
struct CellType {
    uint32_t target_volume, target_interface;
    double lambda_volume, lambda_interface;
};
struct Config {
    int D = 2;
    int grid[3] = {1, 1, 1};
    int periodic = 1;
    int copy_kind = NBH_VON_NEUMANN, energy_kind = NBH_MOORE, conn_kind = NBH_VON_NEUMANN;
    std::vector<CellType> types;
    std::vector<uint64_t> cell_counts;
    std::vector<double> adhesion;  // (n_types+1)^2 row-major, index 0 = medium
    uint64_t seed = 0;
    uint32_t min_cell_volume = 1;
};

// ===========================================================================
// Lattice: lattice.rs:70-255 (halo-padded, row-major, last axis fastest).
// ===========================================================================
struct Lattice {
    int D;
    int64_t dims[3], pdims[3], strides[3];
    bool periodic;
    std::vector<uint32_t> cells;
    void init(int D_, const int* g, bool per) {
        D = D_; periodic = per;
        for (int d = 0; d < 3; ++d) { dims[d] = d < D ? g[d] : 1; pdims[d] = d < D ? g[d] + 2 : 1; }
        int64_t s = 1;
        for (int d = D - 1; d >= 0; --d) { strides[d] = s; s *= pdims[d]; }
        cells.assign((size_t)s, 0);
    }
    int64_t n_sites() const { int64_t n = 1; for (int d = 0; d < D; ++d) n *= dims[d]; return n; }
    int64_t n_padded() const { return (int64_t)cells.size(); }
    int64_t flat(const int64_t* c) const { int64_t f = 0; for (int d = 0; d < D; ++d) f += (c[d] + 1) * strides[d]; return f; }
    void padded_coord(int64_t f, int64_t* pc) const { for (int d = 0; d < D; ++d) { pc[d] = f / strides[d]; f %= strides[d]; } }
    bool is_interior(int64_t f) const {
        for (int d = 0; d < D; ++d) { int64_t c = f / strides[d]; f %= strides[d]; if (c == 0 || c == pdims[d] - 1) return false; }
        return true;
    }
    void interior_coord(int64_t f, int64_t* c) const { padded_coord(f, c); for (int d = 0; d < D; ++d) c[d] -= 1; }
    // lattice.rs:199-220
    int64_t wrapped_interior_flat(int64_t f) const {
        int64_t pc[3], ic[3];
        padded_coord(f, pc);
        for (int d = 0; d < D; ++d) ic[d] = pc[d] == 0 ? dims[d] - 1 : (pc[d] == pdims[d] - 1 ? 0 : pc[d] - 1);
        return flat(ic);
    }
    // lattice.rs:240-254: full halo refresh.
    void refresh_halo() {
        const int64_t n = n_padded();
        for (int64_t f = 0; f < n; ++f) {
            int64_t pc[3];
            padded_coord(f, pc);
            bool halo = false;
            for (int d = 0; d < D; ++d) if (pc[d] == 0 || pc[d] == pdims[d] - 1) halo = true;
            if (!halo) continue;
            cells[f] = cells[wrapped_interior_flat(f)];
        }
    }
    // Same result as refresh_halo() after a single interior site changed:
    // rewrite only the halo cells that mirror it (at most 3^D - 1 of them).
    void refresh_halo_local(int64_t f) {
        int64_t c[3];
        interior_coord(f, c);
        int alt[3][2], na[3];
        for (int d = 0; d < 3; ++d) { na[d] = 1; alt[d][0] = 0; }
        for (int d = 0; d < D; ++d) {
            alt[d][0] = (int)(c[d] + 1);
            na[d] = 1;
            if (c[d] == 0) alt[d][na[d]++] = (int)pdims[d] - 1;
            if (c[d] == dims[d] - 1) alt[d][na[d]++] = 0;
        }
        const uint32_t v = cells[f];
        for (int i0 = 0; i0 < na[0]; ++i0)
            for (int i1 = 0; i1 < (D > 1 ? na[1] : 1); ++i1)
                for (int i2 = 0; i2 < (D > 2 ? na[2] : 1); ++i2) {
                    int64_t g = alt[0][i0] * strides[0];
                    if (D > 1) g += alt[1][i1] * strides[1];
                    if (D > 2) g += alt[2][i2] * strides[2];
                    cells[g] = v;
                }
    }
    template <class F> void each_interior(F fn) const {
        int64_t c[3] = {0, 0, 0};
        const int64_t total = n_sites();
        for (int64_t i = 0; i < total; ++i) {
            fn(c);
            for (int d = D - 1; d >= 0; --d) { if (++c[d] < dims[d]) break; c[d] = 0; }
        }
    }
};

static std::vector<int64_t> offset_table(const std::vector<Off>& st, const Lattice& L) {
    std::vector<int64_t> v;
    for (const Off& o : st) { int64_t d = 0; for (int a = 0; a < L.D; ++a) d += o.c[a] * L.strides[a]; v.push_back(d); }
    return v;
}

// ===========================================================================
// The simulation (model.rs:15-76 + state.rs:168-248).
// ===========================================================================
struct MoveRecord {  // one attempt_at, with the RNG choices supplied
    int64_t target_flat, source_flat;
    uint32_t losing, gaining;
    int32_t null_move;        // losing == gaining
    int32_t topology_ok;      // preserves_topology (true when null or medium)
    int32_t volume_guard_ok;  // !(losing != 0 && V[losing] <= min)
    int32_t evaluated;        // reached the energy computation
    int32_t delta_i_losing, delta_i_gaining;
    double delta_h;
    int32_t accepted;
};

struct Sim {
    Config cfg;
    Lattice lat;
    std::vector<uint32_t> type_of;  // per cell (index id-1)
    std::vector<uint32_t> volume, interface;
    std::vector<int64_t> sum_pos;    // n * D
    std::vector<int64_t> sum_outer;  // n * D * D
    std::vector<uint32_t> contact;   // (n+1)^2, canonical (min,max)
    double energy = 0.0;
    Xoshiro rng;
    uint64_t mcs = 0;
    std::vector<int64_t> copy_off, energy_off, conn_off, topo_off;
    int ntypes = 0;
    bool local_halo = false;
    std::string err;
    // Modes of the same loop: acceptance (monte_carlo.rs:147-196; 0 =
    // Metropolis, 1 = MetropolisHastings) and the Act term
    // (energy.rs:329-471), off unless set.
    int acceptance = 0;
    bool act = false;
    // The connectivity check of an attempt; off only in the reference's
    // exact-Boltzmann harness (`attempt(cpm, false)`, monte_carlo.rs:37-42,
    // tests/exact_boltzmann.rs), where the chain must be free to reshape.
    bool check_topology = true;
    std::vector<double> lambda_act;  // per type
    std::vector<uint32_t> max_act;   // per type
    std::vector<uint32_t> birth;     // per padded site: MCS at which its owner acquired it

    int n_cells() const { return (int)type_of.size(); }
    int type_index_of(uint32_t id) const { return id == 0 ? -1 : (int)type_of[id - 1]; }
    double J(int a, int b) const { return cfg.adhesion[(size_t)a * (ntypes + 1) + b]; }
    int adh(uint32_t id) const { return id == 0 ? 0 : (int)type_of[id - 1] + 1; }

    bool build() {
        ntypes = (int)cfg.types.size();
        lat.init(cfg.D, cfg.grid, cfg.periodic != 0);
        std::vector<Off> s;
        if (!stencil_for(cfg.copy_kind, cfg.D, s)) { err = "bad copy stencil"; return false; }
        copy_off = offset_table(s, lat);
        if (!stencil_for(cfg.energy_kind, cfg.D, s)) { err = "bad energy stencil"; return false; }
        energy_off = offset_table(s, lat);
        if (!stencil_for(cfg.conn_kind, cfg.D, s)) { err = "bad connectivity stencil"; return false; }
        conn_off = offset_table(s, lat);
        topo_off = offset_table(full_moore(cfg.D), lat);
        rng = xoshiro_from_u64(cfg.seed);
        return true;
    }

    // ---- energy.rs:72-115 VolumeTerm / 120-214 InterfaceTerm ----
    double vterm(int t, double v) const {
        const double x = v - (double)cfg.types[t].target_volume;
        return cfg.types[t].lambda_volume * (x * x);
    }
    double iterm(int t, double i) const {
        const double x = i - (double)cfg.types[t].target_interface;
        return cfg.types[t].lambda_interface * (x * x);
    }
    // energy.rs:167-186
    void interface_deltas(int64_t tf, uint32_t lo, uint32_t ga, double& dl, double& dg) const {
        dl = 0.0; dg = 0.0;
        for (int64_t off : energy_off) {
            const uint32_t nc = lat.cells[tf + off];
            dl += nc == lo ? 1.0 : -1.0;
            dg += nc == ga ? -1.0 : 1.0;
        }
    }
    // energy.rs:92-103
    double volume_delta(uint32_t lo, uint32_t ga) const {
        double total = 0.0;
        if (lo) { const int t = type_of[lo - 1]; const double v = volume[lo - 1]; total += vterm(t, v - 1.0) - vterm(t, v); }
        if (ga) { const int t = type_of[ga - 1]; const double v = volume[ga - 1]; total += vterm(t, v + 1.0) - vterm(t, v); }
        return total;
    }
    // energy.rs:190-202
    double interface_delta(int64_t tf, uint32_t lo, uint32_t ga) const {
        double dl, dg;
        interface_deltas(tf, lo, ga, dl, dg);
        double total = 0.0;
        if (lo) { const int t = type_of[lo - 1]; const double i = interface[lo - 1]; total += iterm(t, i + dl) - iterm(t, i); }
        if (ga) { const int t = type_of[ga - 1]; const double i = interface[ga - 1]; total += iterm(t, i + dg) - iterm(t, i); }
        return total;
    }
    // energy.rs:242-264 (weights are all 1.0 after validation, so w*x == x).
    double adhesion_delta(int64_t tf, uint32_t lo, uint32_t ga) const {
        const int li = adh(lo), gi = adh(ga);
        double total = 0.0;
        for (int64_t off : energy_off) {
            const uint32_t nc = lat.cells[tf + off];
            const int ni = adh(nc);
            const double before = nc != lo ? J(li, ni) : 0.0;
            const double after = nc != ga ? J(gi, ni) : 0.0;
            total += 1.0 * (after - before);
        }
        return total;
    }
    // energy.rs:521-523
    double total_delta(int64_t tf, uint32_t lo, uint32_t ga) const {
        return volume_delta(lo, ga) + interface_delta(tf, lo, ga) + adhesion_delta(tf, lo, ga);
    }
    // ---- energy.rs:363-376 canonical_flat, 377-412 geometric_mean ----
    int64_t act_canonical(int64_t f) const { return lat.periodic ? lat.wrapped_interior_flat(f) : f; }
    double act_geometric_mean(int64_t site, uint32_t relevant, uint32_t mx) const {
        const int64_t is = act_canonical(site);
        double product = 1.0;
        uint32_t count = 0;
        auto consider = [&](int64_t f) {
            const int64_t c = act_canonical(f);
            if (lat.cells[c] != relevant) return;
            const uint64_t b = birth[c];
            const uint64_t elapsed = mcs > b ? mcs - b : 0;  // saturating_sub
            const double activity = (double)((uint64_t)mx > elapsed ? (uint64_t)mx - elapsed : 0);
            product *= activity;
            count += 1;
        };
        consider(is);
        for (int64_t off : copy_off) consider(is + off);
        return std::pow(product, 1.0 / (double)count);
    }
    // energy.rs:441-451 ActTerm::delta (0 when the medium gains the site)
    double act_delta(int64_t tf, int64_t sf, uint32_t lo, uint32_t ga) const {
        if (ga == 0) return 0.0;
        const int t = (int)type_of[ga - 1];
        const double lambda = lambda_act[t];
        const uint32_t mx = max_act[t];
        const double gm_src = act_geometric_mean(sf, ga, mx);
        const double gm_tgt = act_geometric_mean(tf, lo, mx);
        return -(lambda / (double)mx) * (gm_src - gm_tgt);
    }
    // monte_carlo.rs:204-224 neighbour_counts over the copy stencil
    void neighbour_counts(int64_t tf, uint32_t lo, uint32_t ga, int& na, int& nb) const {
        na = nb = 0;
        for (int64_t off : copy_off) {
            const uint32_t c = lat.cells[tf + off];
            na += c == lo;
            nb += c == ga;
        }
    }
    // monte_carlo.rs:147-196 decide_acceptance; `draw` yields gen::<f64>()
    // and is called only where the reference draws.
    template <class Draw> bool decide(int64_t tf, uint32_t lo, uint32_t ga, double dh, Draw draw) const {
        if (acceptance == 0) return dh <= 0.0 || draw() < std::exp(-dh);
        int na, nb;
        neighbour_counts(tf, lo, ga, na, nb);
        if (na == 0) return false;
        const double ratio = ((double)na / (double)nb) * std::exp(-dh);
        return draw() < std::fmin(ratio, 1.0);  // f64::min: a NaN operand yields the other
    }

    // energy.rs:104-113, 203-212, 266-308: global energy for the checker.
    double global_energy() const {
        double v = 0.0;
        for (int i = 0; i < n_cells(); ++i) v += vterm(type_of[i], volume[i]);
        double in = 0.0;
        for (int i = 0; i < n_cells(); ++i) in += iterm(type_of[i], interface[i]);
        double a = 0.0;
        lat.each_interior([&](const int64_t* c) {
            const int64_t i = lat.flat(c);
            const uint32_t ic = lat.cells[i];
            const int ii = adh(ic);
            for (int64_t off : energy_off) {
                const int64_t j = i + off;
                int64_t key;
                bool has_key;
                if (lat.is_interior(j)) { key = j; has_key = true; }
                else if (lat.periodic) { key = lat.wrapped_interior_flat(j); has_key = true; }
                else { key = 0; has_key = false; }
                if (has_key && key <= i) continue;
                const uint32_t jc = lat.cells[j];
                if (jc == ic) continue;
                a += 1.0 * J(ii, adh(jc));
            }
        });
        return v + in + a;
    }

    // ---- connectivity.rs:42-65 ----
    uint32_t topo_pattern(int64_t tf, uint32_t lo) const {
        uint32_t p = 0;
        for (size_t i = 0; i < topo_off.size(); ++i)
            if (lat.cells[tf + topo_off[i]] == lo) p |= 1u << i;
        return p;
    }
    bool preserves_topology(int64_t tf, uint32_t lo) const {
        if (lo == 0) return true;
        return checker(cfg.D).is_simple(topo_pattern(tf, lo));
    }

    // ---- dynamics.rs:73-98 ----
    void contact_add(uint32_t a, uint32_t b, int delta) {
        const uint32_t lo = std::min(a, b), hi = std::max(a, b);
        uint32_t& c = contact[(size_t)lo * (n_cells() + 1) + hi];
        if (delta < 0) c = c > 0 ? c - 1 : 0; else c += 1;
    }
    void update_contact(int64_t tf, uint32_t lo, uint32_t ga) {
        if (lo == ga) return;
        for (int64_t off : energy_off) {
            const uint32_t o = lat.cells[tf + off];
            if (o != lo) contact_add(lo, o, -1);
            if (o != ga) contact_add(ga, o, +1);
        }
    }
    // dynamics.rs:106-110
    static uint32_t apply_delta(uint32_t cur, double delta) {
        return (uint32_t)((int64_t)cur + (int64_t)std::round(delta));
    }
    // dynamics.rs:193-202
    static int64_t nearest_image(int64_t coord, double centroid, int64_t extent, bool periodic) {
        if (!periodic) return coord;
        int64_t best = coord;
        double bd = std::fabs((double)coord - centroid);
        const int64_t cand[2] = {coord - extent, coord + extent};
        for (int k = 0; k < 2; ++k) {
            const double dd = std::fabs((double)cand[k] - centroid);
            if (dd < bd) { best = cand[k]; bd = dd; }
        }
        return best;
    }
    // dynamics.rs:125-183 (volume already updated by commit).
    void update_position_sums(int64_t tf, uint32_t lo, uint32_t ga) {
        const int D = cfg.D;
        int64_t c[3];
        lat.interior_coord(tf, c);
        if (lo) {
            const size_t i = lo - 1;
            for (int d = 0; d < D; ++d) sum_pos[i * D + d] -= c[d];
            for (int d = 0; d < D; ++d) for (int e = 0; e < D; ++e) sum_outer[(i * D + d) * D + e] -= c[d] * c[e];
        }
        if (ga) {
            const size_t i = ga - 1;
            uint32_t vb = volume[i] >= 1 ? volume[i] - 1 : 0;
            if (vb < 1) vb = 1;
            double cen[3];
            for (int d = 0; d < D; ++d) cen[d] = (double)sum_pos[i * D + d] / (double)vb;
            int64_t img[3];
            for (int d = 0; d < D; ++d) {
                img[d] = nearest_image(c[d], cen[d], lat.dims[d], lat.periodic);
                sum_pos[i * D + d] += img[d];
            }
            for (int d = 0; d < D; ++d) for (int e = 0; e < D; ++e) sum_outer[(i * D + d) * D + e] += img[d] * img[e];
        }
    }
    // dynamics.rs:206-224
    void refresh_after_commit(int64_t tf) {
        if (!lat.periodic) return;
        int64_t c[3];
        lat.interior_coord(tf, c);
        bool on_b = false;
        for (int d = 0; d < cfg.D; ++d) if (c[d] == 0 || c[d] == lat.dims[d] - 1) on_b = true;
        if (!on_b) return;
        if (local_halo) lat.refresh_halo_local(tf); else lat.refresh_halo();
    }
    // dynamics.rs:23-58 + monte_carlo.rs:226-271
    void commit(int64_t tf, uint32_t lo, uint32_t ga, double dh) {
        double dl, dg;
        interface_deltas(tf, lo, ga, dl, dg);
        update_contact(tf, lo, ga);
        lat.cells[tf] = ga;
        if (lo) { volume[lo - 1] -= 1; interface[lo - 1] = apply_delta(interface[lo - 1], dl); }
        if (ga) { volume[ga - 1] += 1; interface[ga - 1] = apply_delta(interface[ga - 1], dg); }
        update_position_sums(tf, lo, ga);
        refresh_after_commit(tf);
        if (act) birth[tf] = (uint32_t)mcs;  // energy.rs:453-458
        energy += dh;
    }

    // ---- monte_carlo.rs:52-145 with the RNG draws made explicit ----
    // Decides one attempt without mutating anything; `u` is the
    // `gen::<f64>()` draw, consumed only when delta_h > 0.
    void evaluate(int64_t tf, int k, double u, MoveRecord& r) const {
        r = MoveRecord{};
        r.target_flat = tf;
        r.source_flat = tf + copy_off[k];
        r.losing = lat.cells[tf];
        r.gaining = lat.cells[r.source_flat];
        r.null_move = r.losing == r.gaining;
        if (r.null_move) return;
        r.topology_ok = preserves_topology(tf, r.losing);
        if (!r.topology_ok) return;
        r.volume_guard_ok = !(r.losing != 0 && volume[r.losing - 1] <= cfg.min_cell_volume);
        if (!r.volume_guard_ok) return;
        r.evaluated = 1;
        double dl, dg;
        interface_deltas(tf, r.losing, r.gaining, dl, dg);
        r.delta_i_losing = (int32_t)std::round(dl);
        r.delta_i_gaining = (int32_t)std::round(dg);
        r.delta_h = total_delta(tf, r.losing, r.gaining);
        if (act) r.delta_h = r.delta_h + act_delta(tf, r.source_flat, r.losing, r.gaining);
        r.accepted = decide(tf, r.losing, r.gaining, r.delta_h, [u] { return u; });
    }
    bool attempt_at(int64_t tf) {
        const int k = (int)gen_range(rng, 0, copy_off.size());
        const int64_t sf = tf + copy_off[k];
        const uint32_t lo = lat.cells[tf], ga = lat.cells[sf];
        if (lo == ga) return false;
        if (check_topology && !preserves_topology(tf, lo)) return false;
        if (lo != 0 && volume[lo - 1] <= cfg.min_cell_volume) return false;
        const double dh = total_delta(tf, lo, ga);
        // Act steers the decision but never reaches the conservative energy
        // (monte_carlo.rs:82-97)
        const double dh_all = act ? dh + act_delta(tf, sf, lo, ga) : dh;
        const bool acc = decide(tf, lo, ga, dh_all, [this] { return gen_f64(rng); });
        if (acc) commit(tf, lo, ga, dh);
        return acc;
    }
    // monte_carlo.rs:37-42
    bool attempt() {
        int64_t c[3];
        for (int d = 0; d < cfg.D; ++d) c[d] = (int64_t)gen_range(rng, 0, (uint64_t)lat.dims[d]);
        return attempt_at(lat.flat(c));
    }
    // monte_carlo.rs:327-357 (Uniform proposal).
    void run_mcs(uint64_t n) {
        const int64_t ns = lat.n_sites();
        for (uint64_t m = 0; m < n; ++m) {
            for (int64_t i = 0; i < ns; ++i) attempt();
            mcs += 1;
        }
    }

    // ---- initialization.rs:396-436 ----
    void recompute_derived() {
        const int n = n_cells(), D = cfg.D;
        interface.assign(n, 0);
        sum_pos.assign((size_t)n * D, 0);
        sum_outer.assign((size_t)n * D * D, 0);
        lat.each_interior([&](const int64_t* c) {
            const int64_t f = lat.flat(c);
            const uint32_t cell = lat.cells[f];
            if (!cell) return;
            const size_t i = cell - 1;
            for (int d = 0; d < D; ++d) {
                sum_pos[i * D + d] += c[d];
                for (int e = 0; e < D; ++e) sum_outer[(i * D + d) * D + e] += c[d] * c[e];
            }
            for (int64_t off : energy_off) if (lat.cells[f + off] != cell) interface[i] += 1;
        });
        recompute_contact(contact);
    }
    // state.rs:127-157
    void recompute_contact(std::vector<uint32_t>& out) const {
        const int n1 = n_cells() + 1;
        out.assign((size_t)n1 * n1, 0);
        lat.each_interior([&](const int64_t* c) {
            const int64_t i = lat.flat(c);
            const uint32_t ic = lat.cells[i];
            for (int64_t off : energy_off) {
                const int64_t j = i + off;
                int64_t key; bool has;
                if (lat.is_interior(j)) { key = j; has = true; }
                else if (lat.periodic) { key = lat.wrapped_interior_flat(j); has = true; }
                else { key = 0; has = false; }
                if (has && key <= i) continue;
                const uint32_t jc = lat.cells[j];
                if (jc == ic) continue;
                const uint32_t a = std::min(ic, jc), b = std::max(ic, jc);
                out[(size_t)a * n1 + b] += 1;
            }
        });
    }
    // initialization.rs:142-187
    int64_t canonical_neighbour(int64_t f, int64_t off) const {
        const int64_t nb = f + off;
        if (lat.is_interior(nb) || !lat.periodic) return nb;
        return lat.wrapped_interior_flat(nb);
    }
    bool is_connected(uint32_t id) const {
        std::vector<int64_t> sites;
        lat.each_interior([&](const int64_t* c) { const int64_t f = lat.flat(c); if (lat.cells[f] == id) sites.push_back(f); });
        if (sites.empty()) return false;
        std::vector<char> vis(lat.cells.size(), 0);
        std::vector<int64_t> st{sites[0]};
        vis[sites[0]] = 1;
        size_t count = 1;
        while (!st.empty()) {
            const int64_t f = st.back(); st.pop_back();
            for (int64_t off : conn_off) {
                const int64_t nb = canonical_neighbour(f, off);
                if (lat.cells[nb] == id && !vis[nb]) { vis[nb] = 1; ++count; st.push_back(nb); }
            }
        }
        return count == sites.size();
    }
    void finish_init(const std::vector<uint32_t>& vol) {
        volume = vol;
        recompute_derived();
        energy = global_energy();
    }
    // initialization.rs:61-137
    bool place_explicit(const uint32_t* values, int64_t nvals, const uint32_t* cell_type_of, int n) {
        const int64_t ns = lat.n_sites();
        if (nvals != ns) { err = "explicit lattice has " + std::to_string(nvals) + " entries, expected N_sites = " + std::to_string(ns); return false; }
        for (int i = 0; i < n; ++i)
            if ((int)cell_type_of[i] >= ntypes) { err = "cell " + std::to_string(i + 1) + " has type_index " + std::to_string(cell_type_of[i]) + ", but only " + std::to_string(ntypes) + " types are declared"; return false; }
        for (int64_t i = 0; i < nvals; ++i)
            if ((int64_t)values[i] > n) { err = "lattice references cell id " + std::to_string(values[i]) + ", but cell_type_of only covers " + std::to_string(n) + " cells"; return false; }
        std::vector<uint32_t> vol(n, 0);
        int64_t idx = 0;
        lat.each_interior([&](const int64_t* c) {
            const uint32_t v = values[idx++];
            lat.cells[lat.flat(c)] = v;
            if (v) vol[v - 1] += 1;
        });
        if (lat.periodic) lat.refresh_halo();
        for (int i = 0; i < n; ++i)
            if (vol[i] == 0) { err = "cell " + std::to_string(i + 1) + " has zero volume in the supplied lattice"; return false; }
        type_of.assign(cell_type_of, cell_type_of + n);
        for (int id = 1; id <= n; ++id)
            if (!is_connected((uint32_t)id)) { err = "cell " + std::to_string(id) + " is not connected under connectivity_neighborhood"; return false; }
        finish_init(vol);
        return true;
    }
    // initialization.rs:321-333
    double periodic_distance(const int64_t* a, const int64_t* b) const {
        double s = 0.0;
        for (int d = 0; d < cfg.D; ++d) {
            const double raw = std::fabs((double)a[d] - (double)b[d]);
            const double delta = lat.periodic ? std::min(raw, (double)lat.dims[d] - raw) : raw;
            s += delta * delta;
        }
        return std::sqrt(s);
    }
    // initialization.rs:279-318
    bool growable(int64_t f, int64_t off, int64_t& out) const {
        const int64_t raw = f + off;
        if (lat.is_interior(raw) || lat.periodic) { out = canonical_neighbour(f, off); return true; }
        return false;
    }
    // initialization.rs:202-277
    bool scatter_and_grow() {
        std::vector<uint32_t> tcell;
        for (size_t t = 0; t < cfg.cell_counts.size(); ++t)
            for (uint64_t k = 0; k < cfg.cell_counts[t]; ++k) tcell.push_back((uint32_t)t);
        const int n = (int)tcell.size();
        if (n == 0) { err = "cell_counts sums to zero cells — nothing to place"; return false; }
        double avg = 0.0;
        for (const auto& t : cfg.types) avg += (double)t.target_volume;
        avg /= (double)cfg.types.size();
        const double min_sep = std::sqrt(avg / M_PI);
        std::vector<std::array<int64_t, 3>> seeds;
        for (int s = 0; s < n; ++s) {
            bool placed = false;
            for (int a = 0; a < 20000; ++a) {
                std::array<int64_t, 3> cand{0, 0, 0};
                for (int d = 0; d < cfg.D; ++d) cand[d] = (int64_t)gen_range(rng, 0, (uint64_t)lat.dims[d]);
                bool far = true;
                for (auto& q : seeds) if (!(periodic_distance(q.data(), cand.data()) >= min_sep)) { far = false; break; }
                if (far) { seeds.push_back(cand); placed = true; break; }
            }
            if (!placed) {
                char buf[64];
                std::snprintf(buf, sizeof buf, "%.2f", min_sep);
                err = "could not place all " + std::to_string(n) + " seed points with minimum separation " + buf + " — too crowded for this configuration";
                return false;
            }
        }
        std::vector<uint32_t> vol(n, 0);
        for (int i = 0; i < n; ++i) { lat.cells[lat.flat(seeds[i].data())] = (uint32_t)(i + 1); vol[i] += 1; }
        if (lat.periodic) lat.refresh_halo();
        std::vector<uint32_t> target(n);
        for (int i = 0; i < n; ++i) target[i] = cfg.types[tcell[i]].target_volume;
        std::vector<std::vector<int64_t>> frontier(n);
        for (int i = 0; i < n; ++i) {
            const int64_t sf = lat.flat(seeds[i].data());
            for (int64_t off : copy_off) { int64_t nb; if (growable(sf, off, nb) && lat.cells[nb] == 0) frontier[i].push_back(nb); }
        }
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        for (;;) {
            bool grew = false;
            for (int oi = 0; oi < n; ++oi) {
                const int i = order[oi];
                if (vol[i] >= target[i]) continue;
                auto& fr = frontier[i];
                fr.erase(std::remove_if(fr.begin(), fr.end(), [&](int64_t f) { return lat.cells[f] != 0; }), fr.end());
                if (fr.empty()) continue;
                const size_t pick = (size_t)gen_range(rng, 0, fr.size());
                const int64_t claimed = fr[pick];
                fr[pick] = fr.back(); fr.pop_back();  // swap_remove
                lat.cells[claimed] = (uint32_t)(i + 1);
                vol[i] += 1;
                if (lat.periodic) { if (local_halo) lat.refresh_halo_local(claimed); else lat.refresh_halo(); }
                for (int64_t off : copy_off) { int64_t nb; if (growable(claimed, off, nb) && lat.cells[nb] == 0) fr.push_back(nb); }
                grew = true;
            }
            if (!grew) break;
            for (int i = n - 1; i >= 1; --i) {
                const int j = (int)gen_range_incl(rng, 0, (uint64_t)i);
                std::swap(order[i], order[j]);
            }
        }
        type_of = tcell;
        finish_init(vol);
        return true;
    }

    // ---- checker.rs:36-136: brute-force recount vs incremental state ----
    int check(double* energy_rel_err) const {
        const int n = n_cells(), D = cfg.D;
        std::vector<uint32_t> v(n, 0), in(n, 0);
        std::vector<int64_t> sp((size_t)n * D, 0);
        lat.each_interior([&](const int64_t* c) {
            const int64_t f = lat.flat(c);
            const uint32_t cell = lat.cells[f];
            if (!cell) return;
            v[cell - 1] += 1;
            for (int64_t off : energy_off) if (lat.cells[f + off] != cell) in[cell - 1] += 1;
        });
        int bad = 0;
        if (v != volume) bad |= 1;
        if (in != interface) bad |= 2;
        std::vector<uint32_t> ct;
        recompute_contact(ct);
        if (ct != contact) bad |= 4;
        const double g = global_energy();
        const double rel = std::fabs(g - energy) / std::max(1.0, std::fabs(g));
        if (energy_rel_err) *energy_rel_err = rel;
        if (rel > 1e-6) bad |= 8;
        return bad;
    }
};

// ===========================================================================
// Run window (output.rs:147-529) and labelling (labelling.rs:70-154).
// ===========================================================================
struct Labels {
    std::vector<uint32_t> fragmented;
    std::vector<uint32_t> medium_volumes;
    std::vector<uint8_t> medium_touches;
};
static Labels label_components(const Sim& s) {
    const Lattice& L = s.lat;
    Labels out;
    std::vector<char> vis(L.cells.size(), 0);
    std::map<uint32_t, uint32_t> comps;
    const std::vector<int64_t> medium_off = offset_table(full_moore(L.D), L);
    std::deque<int64_t> q;
    auto canonical = [&](int64_t f) -> int64_t {
        if (L.is_interior(f)) return f;
        if (L.periodic) return L.wrapped_interior_flat(f);
        return f;
    };
    L.each_interior([&](const int64_t* c) {
        const int64_t seed = L.flat(c);
        if (vis[seed]) return;
        const uint32_t owner = L.cells[seed];
        const std::vector<int64_t>& offs = owner == 0 ? medium_off : s.conn_off;
        vis[seed] = 1;
        q.push_back(seed);
        uint32_t vol = 0;
        bool touches = false;
        while (!q.empty()) {
            const int64_t site = q.front(); q.pop_front();
            vol += 1;
            for (int64_t off : offs) {
                const int64_t nb = site + off;
                if (!L.is_interior(nb)) {
                    if (owner == 0 && !L.periodic) touches = true;
                    if (!L.periodic) continue;
                }
                const int64_t cn = canonical(nb);
                if (vis[cn]) continue;
                if (L.cells[cn] != owner) continue;
                vis[cn] = 1;
                q.push_back(cn);
            }
        }
        if (owner == 0) { out.medium_volumes.push_back(vol); out.medium_touches.push_back(touches); }
        else comps[owner] += 1;
    });
    for (auto& kv : comps) if (kv.second > 1) out.fragmented.push_back(kv.first);
    return out;
}

// output.rs:183-231
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
    const double p2 = a0 * a0 + a1 * a1 + a2 * a2 + 2.0 * p1;
    const double p = std::sqrt(p2 / 6.0);
    auto b = [&](int i, int j) { const double delta = i == j ? q : 0.0; return (g[i][j] - delta) / p; };
    const double det = b(0, 0) * (b(1, 1) * b(2, 2) - b(1, 2) * b(2, 1))
                     - b(0, 1) * (b(1, 0) * b(2, 2) - b(1, 2) * b(2, 0))
                     + b(0, 2) * (b(1, 0) * b(2, 1) - b(1, 1) * b(2, 0));
    const double r = std::min(1.0, std::max(-1.0, det / 2.0));
    const double phi = std::acos(r) / 3.0;
    const double e1 = q + 2.0 * p * std::cos(phi);
    const double e3 = q + 2.0 * p * std::cos(phi + 2.0 * M_PI / 3.0);
    const double e2 = 3.0 * q - e1 - e3;
    out[0] = e1; out[1] = e2; out[2] = e3;
}
// output.rs:147-178
static void shape_descriptors(int D, const int64_t* outer, uint32_t volume, const double* cen,
                              double* eig, double* rg2, double* kappa2) {
    const double v = (double)volume;
    double g[3][3] = {{0}};
    for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) g[a][b] = (double)outer[a * D + b] / v - cen[a] * cen[b];
    double e[3];
    symmetric_eigenvalues(D, g, e);
    for (int i = 1; i < D; ++i)  // descending, as sort_by(b.partial_cmp(a))
        for (int j = i; j > 0 && e[j] > e[j - 1]; --j) std::swap(e[j], e[j - 1]);
    double sum = 0.0, sq = 0.0;
    for (int i = 0; i < D; ++i) sum += e[i];
    for (int i = 0; i < D; ++i) sq += e[i] * e[i];
    const double d = (double)D;
    *kappa2 = sum > 0.0 ? (d / (d - 1.0)) * (sq / (sum * sum)) - 1.0 / (d - 1.0) : 0.0;
    *rg2 = sum;
    for (int i = 0; i < D; ++i) eig[i] = e[i];
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
    rv /= (double)n;
    const double rs = std::sqrt(rv);
    if (rs == 0.0) return std::fabs(slope) * (double)(n - 1) > 0.0;
    return std::fabs(slope) * (double)(n - 1) > 2.0 * rs;
}

}  // namespace orc

// ===========================================================================
// C API (ctypes).
// ===========================================================================
using namespace orc;

extern "C" {

struct orc_move {
    int64_t target_flat, source_flat;
    uint32_t losing, gaining;
    int32_t null_move, topology_ok, volume_guard_ok, evaluated;
    int32_t delta_i_losing, delta_i_gaining;
    double delta_h;
    int32_t accepted;
    int32_t pad;
};

// Per-cell summary of one sample (output.rs:289-302).
struct orc_cell_sample {
    uint32_t id, volume, interface, pad;
    double centroid[3], eigenvalues[3], rg2, kappa2;
};

void* orc_new(int D, const int* grid, int periodic, int copy_kind, int energy_kind, int conn_kind,
              int n_types, const uint32_t* target_volume, const uint32_t* target_interface,
              const double* lambda_volume, const double* lambda_interface,
              const uint64_t* cell_counts, const double* adhesion, uint64_t seed,
              uint32_t min_cell_volume, char* err, int errlen) {
    Sim* s = new Sim();
    s->cfg.D = D;
    for (int d = 0; d < D; ++d) s->cfg.grid[d] = grid[d];
    s->cfg.periodic = periodic;
    s->cfg.copy_kind = copy_kind; s->cfg.energy_kind = energy_kind; s->cfg.conn_kind = conn_kind;
    for (int t = 0; t < n_types; ++t) {
        s->cfg.types.push_back(CellType{target_volume[t], target_interface[t], lambda_volume[t], lambda_interface[t]});
        s->cfg.cell_counts.push_back(cell_counts ? cell_counts[t] : 0);
    }
    s->cfg.adhesion.assign(adhesion, adhesion + (size_t)(n_types + 1) * (n_types + 1));
    s->cfg.seed = seed;
    s->cfg.min_cell_volume = min_cell_volume;
    if (!s->build()) {
        if (err) std::snprintf(err, errlen, "%s", s->err.c_str());
        delete s;
        return nullptr;
    }
    return s;
}
void orc_free(void* h) { delete (Sim*)h; }
// Act term harness: acquisition MCS per padded site (null keeps it) and the
// completed-MCS counter; the Act delta-H of one proposed copy.
void orc_set_act_state(void* h, const uint32_t* birth, uint64_t mcs) {
    Sim* s = (Sim*)h;
    if (birth && s->act) std::copy(birth, birth + s->birth.size(), s->birth.begin());
    s->mcs = mcs;
}
void orc_get_birth(void* h, uint32_t* out) { Sim* s = (Sim*)h; std::copy(s->birth.begin(), s->birth.end(), out); }
double orc_act_delta(void* h, int64_t target_flat, int64_t source_flat) {
    Sim* s = (Sim*)h;
    return s->act_delta(target_flat, source_flat, s->lat.cells[target_flat], s->lat.cells[source_flat]);
}
// Acceptance (0 Metropolis, 1 MetropolisHastings) and the Act term (null
// lambda_act = off); before the first MCS.
void orc_set_modes(void* h, int acceptance, const double* lambda_act, const uint32_t* max_act) {
    Sim* s = (Sim*)h;
    s->acceptance = acceptance;
    s->act = lambda_act != nullptr;
    if (s->act) {
        s->lambda_act.assign(lambda_act, lambda_act + s->ntypes);
        s->max_act.assign(max_act, max_act + s->ntypes);
        s->birth.assign((size_t)s->lat.n_padded(), 0u);
    }
}
void orc_set_local_halo(void* h, int on) { ((Sim*)h)->local_halo = on != 0; }
void orc_set_check_topology(void* h, int on) { ((Sim*)h)->check_topology = on != 0; }
// checker.rs:151-265: `n` single attempts with the brute-force check after
// every accepted one. Returns the index of the first attempt after which the
// check failed (its mismatch bits in *bad), or -1; *accepted counts accepts.
int64_t orc_attempts_checked(void* h, uint64_t n, uint64_t* accepted, int* bad) {
    Sim* s = (Sim*)h;
    uint64_t acc = 0;
    *bad = 0;
    for (uint64_t a = 0; a < n; ++a) {
        if (!s->attempt()) continue;
        ++acc;
        const int b = s->check(nullptr);
        if (b) { *bad = b; *accepted = acc; return (int64_t)a; }
    }
    *accepted = acc;
    return -1;
}
// Thinned chain samples (tests/exact_boltzmann.rs, single_cell_/two_cell_
// harness): `burn_in` attempts, then per sample `thin` attempts followed by a
// copy of the interior lattice (n_sites words) into out[i * n_sites].
void orc_sample_attempts(void* h, uint64_t burn_in, int64_t n_samples, uint64_t thin, uint32_t* out) {
    Sim* s = (Sim*)h;
    for (uint64_t a = 0; a < burn_in; ++a) s->attempt();
    const int64_t ns = s->lat.n_sites();
    for (int64_t i = 0; i < n_samples; ++i) {
        for (uint64_t a = 0; a < thin; ++a) s->attempt();
        int64_t j = 0;
        s->lat.each_interior([&](const int64_t* c) { out[i * ns + j++] = s->lat.cells[s->lat.flat(c)]; });
    }
}
int orc_init_explicit(void* h, const uint32_t* lattice, int64_t n_sites, const uint32_t* cell_type_of, int n_cells, char* err, int errlen) {
    Sim* s = (Sim*)h;
    if (!s->place_explicit(lattice, n_sites, cell_type_of, n_cells)) { if (err) std::snprintf(err, errlen, "%s", s->err.c_str()); return -1; }
    return 0;
}
int orc_init_default(void* h, char* err, int errlen) {
    Sim* s = (Sim*)h;
    if (!s->scatter_and_grow()) { if (err) std::snprintf(err, errlen, "%s", s->err.c_str()); return -1; }
    return 0;
}
void orc_run_mcs(void* h, uint64_t n) { ((Sim*)h)->run_mcs(n); }
int orc_n_cells(void* h) { return ((Sim*)h)->n_cells(); }
int64_t orc_n_sites(void* h) { return ((Sim*)h)->lat.n_sites(); }
int64_t orc_n_padded(void* h) { return ((Sim*)h)->lat.n_padded(); }
uint64_t orc_mcs(void* h) { return ((Sim*)h)->mcs; }
double orc_energy(void* h) { return ((Sim*)h)->energy; }
double orc_global_energy(void* h) { return ((Sim*)h)->global_energy(); }
void orc_get_volume(void* h, uint32_t* out) { Sim* s = (Sim*)h; std::copy(s->volume.begin(), s->volume.end(), out); }
void orc_get_interface(void* h, uint32_t* out) { Sim* s = (Sim*)h; std::copy(s->interface.begin(), s->interface.end(), out); }
void orc_get_type_of(void* h, uint32_t* out) { Sim* s = (Sim*)h; std::copy(s->type_of.begin(), s->type_of.end(), out); }
void orc_get_sum_position(void* h, int64_t* out) { Sim* s = (Sim*)h; std::copy(s->sum_pos.begin(), s->sum_pos.end(), out); }
void orc_get_sum_outer(void* h, int64_t* out) { Sim* s = (Sim*)h; std::copy(s->sum_outer.begin(), s->sum_outer.end(), out); }
void orc_get_contact(void* h, uint32_t* out) { Sim* s = (Sim*)h; std::copy(s->contact.begin(), s->contact.end(), out); }
void orc_get_padded(void* h, uint32_t* out) { Sim* s = (Sim*)h; std::copy(s->lat.cells.begin(), s->lat.cells.end(), out); }
void orc_get_lattice(void* h, uint32_t* out) {
    Sim* s = (Sim*)h;
    int64_t i = 0;
    s->lat.each_interior([&](const int64_t* c) { out[i++] = s->lat.cells[s->lat.flat(c)]; });
}
void orc_get_strides(void* h, int64_t* out) { Sim* s = (Sim*)h; for (int d = 0; d < 3; ++d) out[d] = s->lat.strides[d]; }
int orc_get_offsets(void* h, int which, int64_t* out) {
    Sim* s = (Sim*)h;
    const std::vector<int64_t>& v = which == 0 ? s->copy_off : which == 1 ? s->energy_off : which == 2 ? s->conn_off : s->topo_off;
    if (out) std::copy(v.begin(), v.end(), out);
    return (int)v.size();
}
int orc_check(void* h, double* rel) { return ((Sim*)h)->check(rel); }
// Overwrite the dynamic state (padded lattice, V, I) for the per-move harness.
void orc_set_state(void* h, const uint32_t* padded, const uint32_t* volume, const uint32_t* interface) {
    Sim* s = (Sim*)h;
    std::copy(padded, padded + s->lat.n_padded(), s->lat.cells.begin());
    std::copy(volume, volume + s->n_cells(), s->volume.begin());
    std::copy(interface, interface + s->n_cells(), s->interface.begin());
}
void orc_evaluate_moves(void* h, int64_t n, const int64_t* target, const int32_t* k, const double* u, orc_move* out) {
    Sim* s = (Sim*)h;
    for (int64_t i = 0; i < n; ++i) {
        MoveRecord r;
        s->evaluate(target[i], k[i], u[i], r);
        orc_move& o = out[i];
        o.target_flat = r.target_flat; o.source_flat = r.source_flat;
        o.losing = r.losing; o.gaining = r.gaining;
        o.null_move = r.null_move; o.topology_ok = r.topology_ok; o.volume_guard_ok = r.volume_guard_ok;
        o.evaluated = r.evaluated; o.delta_i_losing = r.delta_i_losing; o.delta_i_gaining = r.delta_i_gaining;
        o.delta_h = r.delta_h; o.accepted = r.accepted; o.pad = 0;
    }
}
// Apply one accepted move exactly as commit_accepted does (harness helper).
void orc_commit(void* h, int64_t target_flat, uint32_t losing, uint32_t gaining, double delta_h) {
    ((Sim*)h)->commit(target_flat, losing, gaining, delta_h);
}

int orc_is_simple(int D, uint32_t pattern) { return checker(D).is_simple(pattern) ? 1 : 0; }
int orc_slow_is_simple(int D, uint32_t pattern) { return slow_is_simple(D, pattern) ? 1 : 0; }
// Full 3D table (2^26 bits packed into u64 words), as simple_point.rs:344-354.
void orc_table_3d(uint64_t* words) {
    const FastChecker& c = checker(3);
    const uint32_t n = 1u << 26;
    std::memset(words, 0, (n / 64) * sizeof(uint64_t));
    const unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            const uint32_t nw = n / 64;
            for (uint32_t w = t; w < nw; w += nt) {
                uint64_t bits = 0;
                for (uint32_t b = 0; b < 64; ++b) if (c.is_simple(w * 64 + b)) bits |= 1ULL << b;
                words[w] = bits;
            }
        });
    for (auto& x : th) x.join();
}

void orc_blake3(const uint8_t* data, uint64_t len, uint8_t* out32) { b3::hash(data, (size_t)len, out32); }
uint64_t orc_derive_seed_u64(uint64_t master, uint64_t index) { return derive_seed_u64(master, index); }

// Xoshiro stream probe (tests of the RNG restatement itself).
void orc_xoshiro_stream(uint64_t seed, int n, uint64_t* out) { Xoshiro r = xoshiro_from_u64(seed); for (int i = 0; i < n; ++i) out[i] = r.next_u64(); }
void orc_gen_range_stream(uint64_t seed, uint64_t hi, int n, uint64_t* out) { Xoshiro r = xoshiro_from_u64(seed); for (int i = 0; i < n; ++i) out[i] = gen_range(r, 0, hi); }

// Take one sample as output.rs:304-337 does (per-cell summary + labels).
// Returns the number of medium components written (<= max_medium).
int orc_take_sample(void* h, orc_cell_sample* cells, double* energy, uint32_t* fragmented, int* n_fragmented,
                    uint32_t* medium_volumes, uint8_t* medium_touches, int max_medium) {
    Sim* s = (Sim*)h;
    const int D = s->cfg.D;
    for (int i = 0; i < s->n_cells(); ++i) {
        orc_cell_sample& o = cells[i];
        o.id = (uint32_t)(i + 1); o.volume = s->volume[i]; o.interface = s->interface[i]; o.pad = 0;
        for (int d = 0; d < 3; ++d) { o.centroid[d] = 0; o.eigenvalues[d] = 0; }
        for (int d = 0; d < D; ++d) o.centroid[d] = (double)s->sum_pos[(size_t)i * D + d] / (double)s->volume[i];
        shape_descriptors(D, &s->sum_outer[(size_t)i * D * D], s->volume[i], o.centroid, o.eigenvalues, &o.rg2, &o.kappa2);
    }
    *energy = s->energy;
    Labels lab = label_components(*s);
    *n_fragmented = (int)lab.fragmented.size();
    for (size_t i = 0; i < lab.fragmented.size(); ++i) fragmented[i] = lab.fragmented[i];
    int m = std::min<int>(max_medium, (int)lab.medium_volumes.size());
    for (int i = 0; i < m; ++i) { medium_volumes[i] = lab.medium_volumes[i]; medium_touches[i] = lab.medium_touches[i]; }
    return (int)lab.medium_volumes.size();
}

int orc_not_equilibrated(const double* trace, int n) { return not_equilibrated(std::vector<double>(trace, trace + n)) ? 1 : 0; }

// output.rs:456-522: the status of a run from its burn-in energy trace and
// its readout samples, in the reference's order of checks. Samples are given
// as arrays: per sample its MCS, every cell's volume (row k, ids 1..n),
// the first fragmented id (0 none; null = no topology readouts) and, for the
// last sample, the contact pairs with a positive count. kind: 0 Ok,
// 1 NotEquilibrated, 2 Fragmented, 3 CellLost, 4 Degenerate.
int orc_run_status(const double* trace, size_t n_trace, size_t n_samples, const uint64_t* sample_mcs,
                   uint32_t n_cells, const uint32_t* volumes, const uint32_t* first_fragmented,
                   const uint32_t* pairs, size_t n_pairs, uint32_t min_cell_volume, int32_t* kind,
                   uint32_t* cell_id, uint64_t* at_mcs) {
    *kind = 0; *cell_id = 0; *at_mcs = 0;
    // output.rs:459-463: NotEquilibrated from the burn-in trace
    if (not_equilibrated(std::vector<double>(trace, trace + n_trace))) { *kind = 1; return 0; }
    // output.rs:470-485: the first sample with a fragmented cell, its first id
    if (first_fragmented)
        for (size_t k = 0; k < n_samples; ++k)
            if (first_fragmented[k] != 0) {
                *kind = 2; *cell_id = first_fragmented[k]; *at_mcs = sample_mcs[k];
                return 0;
            }
    // output.rs:487-511: a cell at the volume floor over the trailing
    // ceil(0.5 * samples) samples (at least one, at most all)
    {
        size_t window = (size_t)std::ceil((double)n_samples * 0.5);
        window = std::min(std::max(window, (size_t)1), n_samples);
        if (window > 0) {
            const size_t first = n_samples - window;
            for (uint32_t id = 1; id <= n_cells; ++id) {
                bool floor_all = true;
                for (size_t k = first; k < n_samples && floor_all; ++k)
                    floor_all = volumes[k * n_cells + (id - 1)] <= min_cell_volume;
                if (floor_all) { *kind = 3; *cell_id = id; *at_mcs = sample_mcs[first]; return 0; }
            }
        }
    }
    // output.rs:513-522, 531-559: the last sample's cell-adjacency graph
    // (pairs without the medium) is one component holding every cell
    if (first_fragmented && n_samples > 0 && n_cells >= 2) {
        std::map<uint32_t, std::vector<uint32_t>> adj;
        for (size_t q = 0; q < n_pairs; ++q) {
            const uint32_t a = pairs[2 * q], b = pairs[2 * q + 1];
            if (a == 0 || b == 0) continue;
            adj[a].push_back(b);
            adj[b].push_back(a);
        }
        if (!adj.empty()) {
            std::vector<uint32_t> stack{adj.begin()->first};
            std::map<uint32_t, bool> seen{{adj.begin()->first, true}};
            while (!stack.empty()) {
                const uint32_t u = stack.back();
                stack.pop_back();
                for (uint32_t w : adj[u])
                    if (!seen.count(w)) { seen[w] = true; stack.push_back(w); }
            }
            if (seen.size() == n_cells) *kind = 4;
        }
    }
    return 0;
}

void orc_shape_descriptors(int D, const int64_t* outer, uint32_t volume, const double* centroid, double* eig, double* rg2, double* kappa2) {
    shape_descriptors(D, outer, volume, centroid, eig, rg2, kappa2);
}

// Many independent runs of one configuration in parallel (the Rayon
// par_iter of batch.rs:126-152 as a std::thread pool). Seeds come from
// `seeds`; each run does scatter-and-grow (or the shared explicit lattice if
// `explicit_lattice` is non-null), then burn_in + readout MCS, and writes the
// per-cell summary of the LAST sample plus its energy. Returns the number of
// runs that failed to initialise.
int orc_run_many(int D, const int* grid, int periodic, int copy_kind, int energy_kind, int conn_kind,
                 int n_types, const uint32_t* target_volume, const uint32_t* target_interface,
                 const double* lambda_volume, const double* lambda_interface,
                 const uint64_t* cell_counts, const double* adhesion,
                 const uint32_t* explicit_lattice, const uint32_t* explicit_type_of, int explicit_n_cells,
                 int n_runs, const uint64_t* seeds, uint64_t burn_in, uint64_t readout, int threads, int local_halo,
                 int max_cells, orc_cell_sample* out_cells, double* out_energy, int* out_n_cells, int acceptance,
                 const double* lambda_act, const uint32_t* max_act) {
    std::atomic<int> next{0}, failed{0};
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&] {
            for (;;) {
                const int r = next.fetch_add(1);
                if (r >= n_runs) break;
                char err[256];
                Sim* s = (Sim*)orc_new(D, grid, periodic, copy_kind, energy_kind, conn_kind, n_types, target_volume,
                                       target_interface, lambda_volume, lambda_interface, cell_counts, adhesion,
                                       seeds[r], 1, err, sizeof err);
                if (!s) { failed++; out_n_cells[r] = 0; continue; }
                s->local_halo = local_halo != 0;
                orc_set_modes(s, acceptance, lambda_act, max_act);
                bool ok = explicit_lattice
                              ? s->place_explicit(explicit_lattice, s->lat.n_sites(), explicit_type_of, explicit_n_cells)
                              : s->scatter_and_grow();
                if (!ok) { failed++; out_n_cells[r] = 0; delete s; continue; }
                s->run_mcs(burn_in + readout);
                const int n = std::min(max_cells, s->n_cells());
                out_n_cells[r] = n;
                const int Dd = s->cfg.D;
                for (int i = 0; i < n; ++i) {
                    orc_cell_sample& o = out_cells[(size_t)r * max_cells + i];
                    o.id = (uint32_t)(i + 1); o.volume = s->volume[i]; o.interface = s->interface[i]; o.pad = 0;
                    for (int d = 0; d < 3; ++d) { o.centroid[d] = 0; o.eigenvalues[d] = 0; }
                    for (int d = 0; d < Dd; ++d) o.centroid[d] = (double)s->sum_pos[(size_t)i * Dd + d] / (double)s->volume[i];
                    shape_descriptors(Dd, &s->sum_outer[(size_t)i * Dd * Dd], s->volume[i], o.centroid, o.eigenvalues, &o.rg2, &o.kappa2);
                }
                out_energy[r] = s->energy;
                delete s;
            }
        });
    for (auto& x : th) x.join();
    return failed.load();
}

// Independent runs as orc_run_many, each stopped at `n_ckpt` increasing
// cumulative MCS counts along one trajectory (monte_carlo.rs:327-357 run in
// pieces; the chain is the same as one run_mcs call of the total). At each
// checkpoint c of run r: the running energy and every cell's volume and
// interface (rows of max_cells, run-major then checkpoint).
int orc_run_many_checkpoints(int D, const int* grid, int periodic, int copy_kind, int energy_kind, int conn_kind,
                             int n_types, const uint32_t* target_volume, const uint32_t* target_interface,
                             const double* lambda_volume, const double* lambda_interface,
                             const uint64_t* cell_counts, const double* adhesion,
                             const uint32_t* explicit_lattice, const uint32_t* explicit_type_of,
                             int explicit_n_cells, int n_runs, const uint64_t* seeds, int n_ckpt,
                             const uint64_t* ckpt_mcs, int threads, int max_cells, uint32_t* out_volume,
                             uint32_t* out_interface, double* out_energy, int* out_n_cells) {
    std::atomic<int> next{0}, failed{0};
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&] {
            for (;;) {
                const int r = next.fetch_add(1);
                if (r >= n_runs) break;
                char err[256];
                Sim* s = (Sim*)orc_new(D, grid, periodic, copy_kind, energy_kind, conn_kind, n_types, target_volume,
                                       target_interface, lambda_volume, lambda_interface, cell_counts, adhesion,
                                       seeds[r], 1, err, sizeof err);
                if (!s) { failed++; out_n_cells[r] = 0; continue; }
                s->local_halo = true;
                bool ok = explicit_lattice
                              ? s->place_explicit(explicit_lattice, s->lat.n_sites(), explicit_type_of, explicit_n_cells)
                              : s->scatter_and_grow();
                if (!ok) { failed++; out_n_cells[r] = 0; delete s; continue; }
                const int n = std::min(max_cells, s->n_cells());
                out_n_cells[r] = n;
                uint64_t done = 0;
                for (int c = 0; c < n_ckpt; ++c) {
                    s->run_mcs(ckpt_mcs[c] - done);
                    done = ckpt_mcs[c];
                    const size_t row = ((size_t)r * n_ckpt + c) * max_cells;
                    for (int i = 0; i < n; ++i) {
                        out_volume[row + i] = s->volume[i];
                        out_interface[row + i] = s->interface[i];
                    }
                    out_energy[(size_t)r * n_ckpt + c] = s->energy;
                }
                delete s;
            }
        });
    for (auto& x : th) x.join();
    return failed.load();
}

}  // extern "C"
