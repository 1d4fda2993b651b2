// Configuration, validation, theta and the reproducibility hashes.
//
// Error texts follow the reference word for word, because callers match on
// them (tests/python/test_errors.py:8-51): config.rs:287-413,
// cell.rs:40-65, builder.rs:35-96, theta.rs:93-147, batch.rs:26-45.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <thread>

#include "cpm_host.h"

namespace cpmhost {

int64_t n_sites(const Config& c) {
    int64_t n = 1;
    for (int d = 0; d < c.D; ++d) n *= c.grid[d];
    return n;
}

const char* nbh_name(int k) {
    switch (k) {
        case NBH_VON_NEUMANN: return "VonNeumann";
        case NBH_MOORE: return "Moore";
        case NBH_EIGHTEEN: return "Eighteen";
        case NBH_TWENTY_SIX: return "TwentySix";
        default: return "TwentySixWeighted";
    }
}

// neighborhood.rs:45-95: von Neumann = [+e0,-e0,+e1,-e1,(+e2,-e2)]; the full
// shell enumerates base-3 codes with the axis-0 digit fastest.
static std::vector<std::array<int, 3>> full_shell(int D) {
    int total = 1;
    for (int d = 0; d < D; ++d) total *= 3;
    std::vector<std::array<int, 3>> v;
    for (int code = 0; code < total; ++code) {
        int c = code, nz = 0;
        std::array<int, 3> o{0, 0, 0};
        for (int d = 0; d < D; ++d) { o[d] = c % 3 - 1; c /= 3; nz += o[d] != 0; }
        if (nz) v.push_back(o);
    }
    return v;
}

std::vector<std::array<int, 3>> stencil(int kind, int D) {
    std::vector<std::array<int, 3>> v;
    if (kind == NBH_VON_NEUMANN) {
        for (int a = 0; a < D; ++a) {
            std::array<int, 3> p{0, 0, 0}, m{0, 0, 0};
            p[a] = 1; m[a] = -1;
            v.push_back(p); v.push_back(m);
        }
        return v;
    }
    if (kind == NBH_EIGHTEEN) {
        for (auto& o : full_shell(3))
            if ((o[0] != 0) + (o[1] != 0) + (o[2] != 0) <= 2) v.push_back(o);
        return v;
    }
    return full_shell(D);  // Moore (2D), TwentySix (3D), TwentySixWeighted (3D, weighted)
}

// NeighborhoodKind::to_stencil's dimensionality check (neighborhood.rs:179-264).
static std::string stencil_error(int kind, int D) {
    char buf[128];
    if (kind == NBH_MOORE && D != 2) { std::snprintf(buf, sizeof buf, "Moore neighbourhood is 2D only, got D = %d", D); return buf; }
    if (kind == NBH_EIGHTEEN && D != 3) { std::snprintf(buf, sizeof buf, "Eighteen-neighbour is 3D only, got D = %d", D); return buf; }
    if (kind == NBH_TWENTY_SIX && D != 3) { std::snprintf(buf, sizeof buf, "Twenty-six-neighbour is 3D only, got D = %d", D); return buf; }
    if (kind == NBH_TWENTY_SIX_WEIGHTED && D != 3) { std::snprintf(buf, sizeof buf, "Weighted twenty-six-neighbour is 3D only, got D = %d", D); return buf; }
    return "";
}

// Rust's `{}` (Display) of an f64: shortest round-trip digits, positional
// notation, no trailing ".0".
static std::string rust_float(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    char buf[64];
    int p = 1;
    for (; p <= 17; ++p) {
        std::snprintf(buf, sizeof buf, "%.*e", p - 1, x);
        if (std::strtod(buf, nullptr) == x) break;
    }
    std::string s = buf;
    const bool neg = s[0] == '-';
    if (neg) s = s.substr(1);
    const size_t e = s.find('e');
    const int exp = std::atoi(s.c_str() + e + 1);
    std::string digits;
    for (size_t i = 0; i < e; ++i) if (s[i] != '.') digits += s[i];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    std::string out;
    if (exp >= (int)digits.size() - 1) {
        out = digits + std::string(exp - (int)digits.size() + 1, '0');
    } else if (exp >= 0) {
        out = digits.substr(0, exp + 1) + "." + digits.substr(exp + 1);
    } else {
        out = "0." + std::string(-exp - 1, '0') + digits;
    }
    return (neg ? "-" : "") + out;
}

std::string cell_type_error(const CellType& t) {
    if (t.name.empty()) return "cell type name must not be empty";
    const std::pair<const char*, double> checks[3] = {
        {"lambda_volume", t.lambda_volume}, {"lambda_interface", t.lambda_interface}, {"lambda_act", t.lambda_act}};
    for (auto& c : checks)
        if (!std::isfinite(c.second) || c.second < 0.0)
            return std::string(c.first) + " must be finite and non-negative, got " + rust_float(c.second);
    if (t.lambda_act > 0.0 && t.max_act == 0) return "max_act must be positive when lambda_act is positive";
    return "";
}

static std::string grid_debug(const Config& c) {
    std::string s = "[";
    for (int d = 0; d < c.D; ++d) { if (d) s += ", "; s += std::to_string(c.grid[d]); }
    return s + "]";
}

std::string validate(const Config& c) {
    for (int d = 0; d < c.D; ++d)
        if (c.grid[d] == 0) return "every grid dimension must be nonzero, got " + grid_debug(c);
    if (c.conn_nbh != NBH_VON_NEUMANN)
        return std::string("connectivity_neighborhood must be VonNeumann in this version (the simple-point tables only "
                           "support the (4,8)/(6,26) pairing), got ") + nbh_name(c.conn_nbh);
    std::string e = stencil_error(c.copy_nbh, c.D);
    if (!e.empty()) return e;
    e = stencil_error(c.conn_nbh, c.D);
    if (!e.empty()) return e;
    if (c.copy_nbh != NBH_VON_NEUMANN)  // copy must be a subset of the (von Neumann) connectivity stencil
        return std::string("copy_neighborhood ") + nbh_name(c.copy_nbh) + " must be a subset of connectivity_neighborhood " +
               nbh_name(c.conn_nbh);
    e = stencil_error(c.energy_nbh, c.D);
    if (!e.empty()) return e;
    if (c.energy_nbh == NBH_TWENTY_SIX_WEIGHTED)
        return "weighted energy neighbourhoods are not supported yet: interface bookkeeping is integer-typed; use an "
               "unweighted energy_neighborhood (Moore, Eighteen, or TwentySix)";
    if (c.types.empty()) return "at least one cell type is required";
    for (auto& t : c.types) { e = cell_type_error(t); if (!e.empty()) return e; }
    if (c.cell_counts.size() != c.types.size())
        return "cell_counts has " + std::to_string(c.cell_counts.size()) + " entries, expected one per cell type (" +
               std::to_string(c.types.size()) + ")";
    const size_t n1 = c.types.size() + 1;
    bool bad_shape = c.adhesion.size() != n1;
    for (auto& row : c.adhesion) if (row.size() != n1) bad_shape = true;
    if (bad_shape)
        return "adhesion matrix must be " + std::to_string(n1) + "x" + std::to_string(n1) +
               " (n_types + 1 for medium), got " + std::to_string(c.adhesion.size()) + "x" +
               std::to_string(c.adhesion.empty() ? 0 : c.adhesion[0].size());
    for (size_t i = 0; i < n1; ++i)
        for (size_t j = 0; j < n1; ++j) {
            const double a = c.adhesion[i][j], b = c.adhesion[j][i];
            if (!std::isfinite(a))
                return "adhesion[" + std::to_string(i) + "][" + std::to_string(j) + "] = " + rust_float(a) + " is not finite";
            if (std::fabs(a - b) > 0.0)
                return "adhesion matrix must be symmetric in v1: [" + std::to_string(i) + "][" + std::to_string(j) +
                       "] = " + rust_float(a) + " but [" + std::to_string(j) + "][" + std::to_string(i) + "] = " + rust_float(b);
        }
    if (c.readout == 0) return "readout_mcs must be positive";
    if (c.interval == 0) return "sampling_interval_mcs must be positive";
    if (c.proposal == PROP_EDGE_LIST && c.acceptance == ACC_METROPOLIS_HASTINGS)
        return "proposal = EdgeList is not valid with acceptance = MetropolisHastings: the exact-Boltzmann validation's "
               "reversibility argument depends on the uniform proposal's forward/reverse symmetry, which EdgeList does "
               "not establish";
    return "";
}

// ------------------------------------------------------------------ theta ----
size_t theta_len(size_t n) { return n + n + (n + 1) * (n + 2) / 2 + n + n; }

std::vector<double> theta_extract(const Config& c) {
    const size_t n = c.types.size();
    std::vector<double> th;
    for (auto& t : c.types) th.push_back(t.lambda_volume);
    for (auto& t : c.types) th.push_back(t.lambda_interface);
    for (size_t i = 0; i <= n; ++i)
        for (size_t j = i; j <= n; ++j) th.push_back(c.adhesion[i][j]);
    for (auto& t : c.types) th.push_back(t.lambda_act);
    for (auto& t : c.types) th.push_back((double)t.max_act);
    return th;
}

std::vector<std::string> theta_names(const Config& c) {
    const size_t n = c.types.size();
    auto label = [&](size_t i) { return i == 0 ? std::string("medium") : c.types[i - 1].name; };
    std::vector<std::string> v;
    for (auto& t : c.types) v.push_back("lambda_volume[" + t.name + "]");
    for (auto& t : c.types) v.push_back("lambda_interface[" + t.name + "]");
    for (size_t i = 0; i <= n; ++i)
        for (size_t j = i; j <= n; ++j) v.push_back("J[" + label(i) + "][" + label(j) + "]");
    for (auto& t : c.types) v.push_back("lambda_act[" + t.name + "]");
    for (auto& t : c.types) v.push_back("max_act[" + t.name + "]");
    return v;
}

std::string theta_inject(Config& c, const double* th) {
    const size_t n = c.types.size();
    const size_t len = theta_len(n);
    for (size_t i = 0; i < n; ++i) {
        const double v = th[len - n + i];
        const double r = std::round(v);
        if (!std::isfinite(r) || r < 0.0 || r > 4294967295.0)
            return "max_act[" + c.types[i].name + "] = " + rust_float(v) +
                   " does not round to a value representable as u32 (must be finite and within [0, 4294967295])";
    }
    size_t k = 0;
    for (auto& t : c.types) t.lambda_volume = th[k++];
    for (auto& t : c.types) t.lambda_interface = th[k++];
    for (size_t i = 0; i <= n; ++i)
        for (size_t j = i; j <= n; ++j) { c.adhesion[i][j] = th[k]; c.adhesion[j][i] = th[k]; ++k; }
    for (auto& t : c.types) t.lambda_act = th[k++];
    for (auto& t : c.types) t.max_act = (uint32_t)std::round(th[k++]);
    return "";
}

// ----------------------------------------------------------------- BLAKE3 ----
// The published BLAKE3 construction: 7-round compression over 64-byte
// blocks, 1024-byte chunks, and a binary tree whose left subtree always holds
// the largest power-of-two number of chunks.
namespace {
const uint32_t B3_IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                           0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
const uint8_t B3_SIGMA[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
inline uint32_t ror(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
inline void qr(uint32_t* v, int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] += v[b] + x; v[d] = ror(v[d] ^ v[a], 16); v[c] += v[d]; v[b] = ror(v[b] ^ v[c], 12);
    v[a] += v[b] + y; v[d] = ror(v[d] ^ v[a], 8);  v[c] += v[d]; v[b] = ror(v[b] ^ v[c], 7);
}
void b3_compress(const uint32_t h[8], const uint8_t* blk, uint32_t blen, uint64_t ctr, uint32_t flags, uint32_t out[8]) {
    uint32_t m[16];
    uint8_t buf[64] = {0};
    std::memcpy(buf, blk, blen);
    for (int i = 0; i < 16; ++i) m[i] = buf[4 * i] | (buf[4 * i + 1] << 8) | (buf[4 * i + 2] << 16) | ((uint32_t)buf[4 * i + 3] << 24);
    uint32_t v[16] = {h[0], h[1], h[2], h[3], h[4], h[5], h[6], h[7], B3_IV[0], B3_IV[1], B3_IV[2], B3_IV[3],
                      (uint32_t)ctr, (uint32_t)(ctr >> 32), blen, flags};
    for (int r = 0; r < 7; ++r) {
        qr(v, 0, 4, 8, 12, m[0], m[1]);   qr(v, 1, 5, 9, 13, m[2], m[3]);
        qr(v, 2, 6, 10, 14, m[4], m[5]);  qr(v, 3, 7, 11, 15, m[6], m[7]);
        qr(v, 0, 5, 10, 15, m[8], m[9]);  qr(v, 1, 6, 11, 12, m[10], m[11]);
        qr(v, 2, 7, 8, 13, m[12], m[13]); qr(v, 3, 4, 9, 14, m[14], m[15]);
        uint32_t t[16];
        for (int i = 0; i < 16; ++i) t[i] = m[B3_SIGMA[i]];
        std::memcpy(m, t, sizeof m);
    }
    for (int i = 0; i < 8; ++i) out[i] = v[i] ^ v[i + 8];
}
void b3_chunk(const uint8_t* p, size_t n, uint64_t idx, bool root, uint32_t out[8]) {
    uint32_t h[8];
    std::memcpy(h, B3_IV, sizeof h);
    const size_t nb = n == 0 ? 1 : (n + 63) / 64;
    for (size_t b = 0; b < nb; ++b) {
        const size_t off = b * 64, len = n > off ? (n - off < 64 ? n - off : 64) : 0;
        uint32_t f = (b == 0 ? 1u : 0u) | (b + 1 == nb ? (2u | (root ? 8u : 0u)) : 0u);
        b3_compress(h, p + off, (uint32_t)len, idx, f, h);
    }
    std::memcpy(out, h, 32);
}
// Subtrees of at least this many chunks split their halves over two threads
// (up to `spawn` levels deep): the tree's halves are independent.
constexpr uint64_t B3_PAR_CHUNKS = 512;

void b3_tree(const uint8_t* data, size_t len, uint64_t first, uint64_t count, bool root, uint32_t out[8],
             int spawn = 0) {
    if (count == 1) {
        const size_t off = first * 1024;
        b3_chunk(data + off, len - off < 1024 ? len - off : 1024, first, root, out);
        return;
    }
    uint64_t left = 1;
    while (left * 2 < count) left *= 2;
    uint32_t l[8], r[8];
    if (spawn > 0 && count >= B3_PAR_CHUNKS) {
        std::thread t([&] { b3_tree(data, len, first, left, false, l, spawn - 1); });
        b3_tree(data, len, first + left, count - left, false, r, spawn - 1);
        t.join();
    } else {
        b3_tree(data, len, first, left, false, l, spawn);
        b3_tree(data, len, first + left, count - left, false, r, spawn);
    }
    uint8_t blk[64];
    for (int i = 0; i < 8; ++i)
        for (int b = 0; b < 4; ++b) { blk[4 * i + b] = (uint8_t)(l[i] >> (8 * b)); blk[32 + 4 * i + b] = (uint8_t)(r[i] >> (8 * b)); }
    b3_compress(B3_IV, blk, 64, 0, 4u | (root ? 8u : 0u), out);
}
}  // namespace

void blake3(const uint8_t* data, size_t len, uint8_t out[32]) {
    uint32_t h[8];
    int spawn = 0;
    for (unsigned hw = std::thread::hardware_concurrency(); hw > 1 && spawn < 5; hw >>= 1) ++spawn;
    b3_tree(data, len, 0, len == 0 ? 1 : (len + 1023) / 1024, true, h, spawn);
    for (int i = 0; i < 8; ++i)
        for (int b = 0; b < 4; ++b) out[4 * i + b] = (uint8_t)(h[i] >> (8 * b));
}

// rng.rs:20-40
uint64_t derive_seed_u64(uint64_t master, uint64_t index) {
    uint8_t in[16], out[32];
    for (int i = 0; i < 8; ++i) { in[i] = (uint8_t)(master >> (8 * i)); in[8 + i] = (uint8_t)(index >> (8 * i)); }
    blake3(in, 16, out);
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)out[i] << (8 * i);
    return v;
}

// ----------------------------------------------------------- serde_json ----
static void json_str(std::string& o, const std::string& s) {
    static const char* hex = "0123456789abcdef";
    o += '"';
    for (unsigned char ch : s) {
        switch (ch) {
            case '"': o += "\\\""; break;
            case '\\': o += "\\\\"; break;
            case '\n': o += "\\n"; break;
            case '\r': o += "\\r"; break;
            case '\t': o += "\\t"; break;
            case 0x08: o += "\\b"; break;
            case 0x0c: o += "\\f"; break;
            default:
                if (ch < 0x20) { o += "\\u00"; o += hex[ch >> 4]; o += hex[ch & 15]; }
                else o += (char)ch;
        }
    }
    o += '"';
}
// Decimal digits of x at q; returns the end.
static inline char* put_uint(char* q, uint64_t x) {
    static const struct Pairs {
        char d[200];
        Pairs() { for (int i = 0; i < 100; ++i) { d[2 * i] = (char)('0' + i / 10); d[2 * i + 1] = (char)('0' + i % 10); } }
    } P;
    char tmp[20];
    int k = 20;
    while (x >= 100) {
        const unsigned r = (unsigned)(x % 100);
        x /= 100;
        k -= 2;
        std::memcpy(tmp + k, P.d + 2 * r, 2);
    }
    if (x >= 10) { k -= 2; std::memcpy(tmp + k, P.d + 2 * x, 2); }
    else tmp[--k] = (char)('0' + x);
    std::memcpy(q, tmp + k, (size_t)(20 - k));
    return q + (20 - k);
}

// A JSON array of unsigned integers; large arrays are formatted in parallel
// segments and joined.
template <class T>
static void json_uints(std::string& o, const std::vector<T>& v) {
    const size_t n = v.size();
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t parts = n >= (1u << 17) ? std::min<size_t>(hw, n >> 15) : 1;
    std::vector<std::string> seg(parts);
    auto fmt = [&](size_t p) {
        const size_t a = n * p / parts, b = n * (p + 1) / parts;
        std::string& s = seg[p];
        s.resize((b - a) * 21);
        char* q = &s[0];
        for (size_t i = a; i < b; ++i) {
            if (i) *q++ = ',';
            q = put_uint(q, (uint64_t)v[i]);
        }
        s.resize((size_t)(q - s.data()));
    };
    std::vector<std::thread> th;
    for (size_t p = 1; p < parts; ++p) th.emplace_back(fmt, p);
    fmt(0);
    for (auto& t : th) t.join();
    size_t len = 2;
    for (auto& s : seg) len += s.size();
    o.reserve(o.size() + len);
    o += '[';
    for (auto& s : seg) o += s;
    o += ']';
}
static std::string hex32(const uint8_t d[32]) {
    static const char* h = "0123456789abcdef";
    std::string s;
    for (int i = 0; i < 32; ++i) { s += h[d[i] >> 4]; s += h[d[i] & 15]; }
    return s;
}

// ConventionView, fields in declaration order (config.rs:430-461).
std::string convention_hash(const Config& c) {
    std::string o = "{\"dimensionality\":" + std::to_string(c.D) + ",\"grid\":[";
    for (int d = 0; d < c.D; ++d) { if (d) o += ','; o += std::to_string(c.grid[d]); }
    o += "],\"copy_neighborhood\":{\"kind\":\"" + std::string(nbh_name(c.copy_nbh)) + "\"}";
    o += ",\"energy_neighborhood\":{\"kind\":\"" + std::string(nbh_name(c.energy_nbh)) + "\"}";
    o += ",\"connectivity_neighborhood\":{\"kind\":\"" + std::string(nbh_name(c.conn_nbh)) + "\"}";
    o += std::string(",\"boundary\":\"") + (c.periodic ? "Periodic" : "Fixed") + "\"";
    o += std::string(",\"acceptance\":\"") + (c.acceptance == ACC_METROPOLIS ? "Metropolis" : "MetropolisHastings") + "\"";
    o += std::string(",\"proposal\":\"") + (c.proposal == PROP_UNIFORM ? "Uniform" : "EdgeList") + "\"";
    o += ",\"cell_types\":[";
    for (size_t i = 0; i < c.types.size(); ++i) {
        if (i) o += ',';
        o += "{\"name\":";
        json_str(o, c.types[i].name);
        o += ",\"target_volume\":" + std::to_string(c.types[i].target_volume) +
             ",\"target_interface\":" + std::to_string(c.types[i].target_interface) + "}";
    }
    o += "],\"active_terms\":{";
    o += std::string("\"volume\":") + (c.active.volume ? "true" : "false");
    o += std::string(",\"interface\":") + (c.active.interface ? "true" : "false");
    o += std::string(",\"adhesion\":") + (c.active.adhesion ? "true" : "false");
    o += std::string(",\"act\":") + (c.active.act ? "true" : "false") + "}";
    o += ",\"initialization\":";
    if (c.init_explicit) {
        o += "{\"Explicit\":{\"lattice\":";
        json_uints(o, c.init_lattice);
        o += ",\"cell_type_of\":";
        json_uints(o, c.init_type_of);
        o += "}}";
    } else {
        o += std::string("{\"Default\":{\"warn_on_default_init\":") + (c.warn_on_default_init ? "true" : "false") + "}}";
    }
    o += ",\"burn_in_mcs\":" + std::to_string(c.burn_in) + ",\"readout_mcs\":" + std::to_string(c.readout) +
         ",\"sampling_interval_mcs\":" + std::to_string(c.interval) +
         ",\"min_cell_volume\":" + std::to_string(c.min_cell_volume) +
         ",\"seed_policy\":\"Independent\",\"requested_readouts\":[],\"convention_version\":1}";
    uint8_t d[32];
    blake3((const uint8_t*)o.data(), o.size(), d);
    return hex32(d);
}

// ModelHashView (config.rs:463-556).
std::string model_hash(const Config& c, const std::vector<uint32_t>& lattice, const std::vector<uint32_t>& type_of) {
    return model_hash_with(convention_hash(c), lattice, type_of);
}

std::string model_hash_with(const std::string& conv, const std::vector<uint32_t>& lattice,
                            const std::vector<uint32_t>& type_of) {
    std::string o = "{\"convention_hash\":\"" + conv + "\",\"lattice\":";
    json_uints(o, lattice);
    o += ",\"cell_type_of\":";
    json_uints(o, type_of);
    o += "}";
    uint8_t d[32];
    blake3((const uint8_t*)o.data(), o.size(), d);
    return hex32(d);
}

}  // namespace cpmhost
