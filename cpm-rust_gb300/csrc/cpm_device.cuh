// Device-side building blocks of the Cellular Potts hot path (sm_103a).
//
// Restates, on the GPU, the per-attempt logic of the reference
// (crates/cpm-core/src/monte_carlo.rs:52-145): the early-out, the
// simple-point connectivity test (connectivity.rs:42-65), the volume guard
// (monte_carlo.rs:77-79), the local Delta-H in FP64 with the reference's
// operation order (energy.rs:92-103, 167-202, 242-264, 521-523) and the
// commit bookkeeping (dynamics.rs:23-183). Random numbers come from a
// counter-based Philox4x32-10 (Salmon et al., "Parallel random numbers: as
// easy as 1, 2, 3", SC'11), so every attempt's draws are a pure function of
// (seed, mcs, site) and independent of scheduling.
#pragma once
#include <stdint.h>
#include "cpm_common.h"

namespace cpmgpu {

// ---------------------------------------------------------------- Philox ----
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

enum : uint32_t { TAG_SITE = 0u, TAG_ORDER = 1u, TAG_PASS = 2u };

// Draws of one site attempt at one MCS: x -> copy direction, (z,w) -> u.
__device__ __forceinline__ uint4 site_draw(uint64_t seed, uint64_t mcs, uint32_t site) {
    return philox4x32_10(make_uint4(site, (uint32_t)mcs, (uint32_t)(mcs >> 32) ^ (TAG_SITE << 28), 0x43504D31u),
                         (uint32_t)seed, (uint32_t)(seed >> 32));
}
__device__ __forceinline__ uint4 aux_draw(uint64_t seed, uint64_t mcs, uint32_t tag, uint32_t a, uint32_t b) {
    return philox4x32_10(make_uint4(a, (uint32_t)mcs, (uint32_t)(mcs >> 32) ^ (tag << 28), b),
                         (uint32_t)seed, (uint32_t)(seed >> 32));
}
// 53-bit uniform in [0,1), same resolution as rand's gen::<f64>().
__device__ __forceinline__ double u53(uint4 r) {
    const uint64_t v = (((uint64_t)r.z << 32) | r.w) >> 11;
    return __dmul_rn((double)v, 1.0 / 9007199254740992.0);  // times 2^-53: exact
}
// Priority hash for the conflict-resolution order (murmur3 finaliser).
__device__ __forceinline__ uint32_t mix32(uint32_t h) {
    h ^= h >> 16; h *= 0x85EBCA6Bu;
    h ^= h >> 13; h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// ------------------------------------------------------ simple points ----
// 2D: the 256-entry table (simple_point.rs:288-306) as 8 words.
__device__ __forceinline__ bool table2d_bit(const uint32_t* t2, uint32_t p) {
    return (t2[p >> 5] >> (p & 31u)) & 1u;
}
// 3D: the 2^26-bit table (simple_point.rs:337-366), L2-resident in HBM.
__device__ __forceinline__ bool table3d_bit(const uint64_t* t3, uint32_t p) {
    return (__ldg(t3 + (p >> 6)) >> (p & 63u)) & 1ull;
}

template <int D, class SigT>
__device__ __forceinline__ bool preserves_topology(const SimDesc& s, const SigT* sig, int64_t t, uint32_t losing,
                                                   const uint32_t* t2, const uint64_t* t3) {
    if (losing == 0) return true;  // medium is exempt (connectivity.rs:48-50)
    constexpr int NF = D == 2 ? 8 : 26;
    uint32_t p = 0;
#pragma unroll
    for (int i = 0; i < NF; ++i) p |= (uint32_t)((uint32_t)sig[t + s.topo_off[i]] == losing) << i;
    return D == 2 ? table2d_bit(t2, p) : table3d_bit(t3, p);
}

// True when every copy neighbour of t holds `id` (= sigma[t]): the attempt
// at t is null (monte_carlo.rs:60-64) for every copy direction, so a sweep
// can skip its draw; draws are counters of (seed, MCS, site), so skipping
// one changes no other.
template <class SigT>
__device__ __forceinline__ bool copy_uniform(const SimDesc& s, const SigT* sig, int64_t t, uint32_t id) {
    bool u = true;
    for (int k = 0; k < s.n_copy; ++k) u &= (uint32_t)sig[t + s.copy_off[k]] == id;
    return u;
}

// ------------------------------------------------------------ Delta-H ----
// term(t, x) = lambda[t] * (x - target[t])^2, powi(2) == x*x (energy.rs:85-88).
__device__ __forceinline__ double quad_term(double lambda, uint32_t target, double x) {
    const double d = __dsub_rn(x, (double)target);
    return __dmul_rn(lambda, __dmul_rn(d, d));
}

struct DeltaOut {
    double dh;
    int dl, dg;  // integer interface deltas (every weight is 1.0)
};

// lambda * (x - target)^2 for an integer-valued x: the exact host-built
// table when x is in range (same IEEE operations), else computed here.
__device__ __forceinline__ double term_of(const double* tab, int tab_n, int ty, const double* lambda,
                                          const uint32_t* target, int64_t x) {
    if (tab != nullptr && x >= 0 && x < tab_n) return tab[(int64_t)ty * tab_n + x];
    return quad_term(lambda[ty], target[ty], (double)x);
}

// Terms::total_delta = volume + interface + adhesion, each accumulated in the
// reference's order (energy.rs:92-103, 190-202, 242-264, 521-523). Every
// operation is the reference's f64 operation, rounded to nearest, never
// fused: explicit _rn intrinsics, and the tables hold values computed with
// the same operations on the host. Adding a zero to the running sums is
// skipped: a sum that starts at +0.0 can never become -0.0 under
// round-to-nearest, so x + (+-0.0) == x bit for bit.
template <int NE, class SigT>
__device__ __forceinline__ DeltaOut delta_h(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                            const uint32_t* volume, const uint32_t* interface, int64_t t,
                                            uint32_t L, uint32_t G) {
    const int nt1 = s.n_types + 1;
    const int li = adh_of[L], gi = adh_of[G];
    double adh = 0.0;
    int cl = 0, cg = 0;
    if (s.dj != nullptr) {
        const double* D = s.dj + (int64_t)(li * nt1 + gi) * nt1;
        const double jgl = s.J[gi * nt1 + li];   // neighbour == losing: after - 0.0
        const double jlg = -s.J[li * nt1 + gi];  // neighbour == gaining: 0.0 - before
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const uint32_t nc = (uint32_t)sig[t + s.energy_off[k]];
            const bool isl = nc == L, isg = nc == G;
            cl += isl;
            cg += isg;
            const double d = isl ? jgl : (isg ? jlg : D[adh_of[nc]]);
            adh = __dadd_rn(adh, d);
        }
    } else {
        const double* JL = s.J + li * nt1;
        const double* JG = s.J + gi * nt1;
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const uint32_t nc = (uint32_t)sig[t + s.energy_off[k]];
            cl += nc == L;
            cg += nc == G;
            const int ni = adh_of[nc];
            const double before = nc != L ? JL[ni] : 0.0;
            const double after = nc != G ? JG[ni] : 0.0;
            adh = __dadd_rn(adh, __dsub_rn(after, before));  // w == 1.0: w*x == x
        }
    }
    DeltaOut o;
    o.dl = 2 * cl - NE;  // sum_k (n == L ? +1 : -1)
    o.dg = NE - 2 * cg;  // sum_k (n == G ? -1 : +1)
    double vol = 0.0, itf = 0.0;
    if (L) {
        const int ty = li - 1;
        const int64_t v = volume[L];
        vol = __dadd_rn(vol, __dsub_rn(term_of(s.vterm, s.tab_n, ty, s.lambda_v, s.target_v, v - 1),
                                       term_of(s.vterm, s.tab_n, ty, s.lambda_v, s.target_v, v)));
    }
    if (G) {
        const int ty = gi - 1;
        const int64_t v = volume[G];
        vol = __dadd_rn(vol, __dsub_rn(term_of(s.vterm, s.tab_n, ty, s.lambda_v, s.target_v, v + 1),
                                       term_of(s.vterm, s.tab_n, ty, s.lambda_v, s.target_v, v)));
    }
    if (L) {
        const int ty = li - 1;
        const int64_t i = interface[L];
        itf = __dadd_rn(itf, __dsub_rn(term_of(s.iterm, s.tab_n, ty, s.lambda_i, s.target_i, i + o.dl),
                                       term_of(s.iterm, s.tab_n, ty, s.lambda_i, s.target_i, i)));
    }
    if (G) {
        const int ty = gi - 1;
        const int64_t i = interface[G];
        itf = __dadd_rn(itf, __dsub_rn(term_of(s.iterm, s.tab_n, ty, s.lambda_i, s.target_i, i + o.dg),
                                       term_of(s.iterm, s.tab_n, ty, s.lambda_i, s.target_i, i)));
    }
    o.dh = __dadd_rn(__dadd_rn(vol, itf), adh);
    return o;
}

// Metropolis arm of decide_acceptance (monte_carlo.rs:158):
// dh <= 0 || u < exp(-dh), with exp the FP64 exponential. The FP64 exp is
// only evaluated near the decision threshold: expf(x) has at most 2 ulp
// error (relative 2.4e-7), rounding -dh to float moves exp by at most
// |dh| * 2^-24 relative (<= 3.9e-6 for dh <= 64), and rounding u to float
// 2^-24; a relative band of 2e-5 around expf therefore contains the exact
// threshold, and outside the band the FP32 comparison gives the FP64 answer.
// For dh > 64, exp(-dh) < 1.7e-28 while u is 0 or >= 2^-53.
__device__ __forceinline__ bool metropolis(double dh, double u) {
    if (dh <= 0.0) return true;
    if (dh > 64.0) {
        if (u > 1e-20) return false;
        return u < exp(-dh);
    }
    const float ef = expf(-(float)dh);
    const float uf = (float)u;
    if (uf < ef * 0.99998f) return true;
    if (uf > ef * 1.00002f) return false;
    return u < exp(-dh);
}

// ------------------------------------------------- bounded decision ----
// decide_move returns the reference's Metropolis decision for one attempt
// (monte_carlo.rs:77-82, 158) without FP64 arithmetic in the common case.
//
// Delta-H is first summed in float. Its leaves are the FP64 values the
// reference adds: the adhesion differences and J entries (x = after -
// before), converted y = fl32(x), and the four term differences
// term(x') - term(x), each formed as (c_hi - d_hi) + (c_lo - d_lo) from the
// float pairs of the two FP64 table entries, which is within
// 2 u32 |leaf| + 2^-46 (|c| + |d|) of the FP64 difference. Both the float
// and the reference's FP64 sums are trees of height h <= NE + 3 <= 29 over
// these leaves, so (Higham, "Accuracy and Stability of Numerical
// Algorithms", 2nd ed., sec. 4.2)
//   |dh32 - dh64| <= (gamma32_h + 3 u32) sum|leaf| + 2^-45 sum(|c| + |d|)
//                 <= 1.9e-6 sum|leaf| + 3e-14 sum(|c| + |d|),
// u32 = 2^-24, gamma_h = h u / (1 - h u). The code uses
// eps = 4e-6 sum|leaf| + 1e-12 sum(|c| + |d|), which also covers the float
// rounding of the sums themselves and of dh32 +- eps. Then:
// `draw` supplies the attempt's uniform u (u()) and its top 32 bits
// z = floor(u 2^32) (z()), computed only when needed.
struct PhiloxDraw {  // the sweeps: Philox keyed by (seed, mcs, site)
    uint64_t seed, mcs;
    uint32_t site;
    __device__ double u() const { return u53(site_draw(seed, mcs, site)); }
    __device__ uint32_t z() const { return site_draw(seed, mcs, site).z; }
};
struct GivenDraw {  // the parity harness: u given
    double u_;
    __device__ double u() const { return u_; }
    __device__ uint32_t z() const { return (uint32_t)__dmul_rn(u_, 4294967296.0); }
};

// The two halves of decide_move. The neighbour half depends on sigma only
// (the target's energy neighbours, never written by another attempt of the
// same colour pass), the cell half on the volumes and interfaces of the two
// cells; a caller that has run the neighbour half once re-runs only the
// cell half when those cells change. Together they are decide_move, with
// the same float operations in the same order.
struct NeighbourPart {
    float adh, sabs;  // float adhesion sum over the neighbours, sum of |leaf|
    int dl, dg;       // integer interface deltas
    bool fast;        // float tables present (else the FP64 path decides)
};

template <int NE, class SigT, class Off>
__device__ __forceinline__ NeighbourPart decide_neighbours(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                                           const Off* energy_off, int64_t t, uint32_t L, uint32_t G) {
    const int nt1 = s.n_types + 1;
    const int li = adh_of[L], gi = adh_of[G];
    NeighbourPart o;
    o.fast = s.dj32 != nullptr;
    float adh = 0.f, sabs = 0.f;
    int cl = 0, cg = 0;
    if (o.fast) {
        const float* Dt = s.dj32 + (li * nt1 + gi) * nt1;
        const float jgl = s.J32[gi * nt1 + li];
        const float jlg = -s.J32[li * nt1 + gi];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const uint32_t nc = (uint32_t)sig[t + energy_off[k]];
            const bool isl = nc == L, isg = nc == G;
            cl += isl;
            cg += isg;
            const float d = isl ? jgl : (isg ? jlg : Dt[adh_of[nc]]);
            adh += d;
            sabs += fabsf(d);
        }
    } else {
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const uint32_t nc = (uint32_t)sig[t + energy_off[k]];
            cl += nc == L;
            cg += nc == G;
        }
    }
    o.adh = adh;
    o.sabs = sabs;
    o.dl = 2 * cl - NE;
    o.dg = NE - 2 * cg;
    return o;
}

// The cell half: 1 = accept, 0 = reject, -1 = the float bracket cannot
// decide (the caller then runs the FP64 computation in the reference's
// order). `li` / `gi` are the adhesion indices (type + 1) of L and G.
template <class Draw>
__device__ __forceinline__ int decide_cells(const SimDesc& s, const NeighbourPart& nb, int li, int gi,
                                            const uint32_t* volume, const uint32_t* interface, uint32_t L,
                                            uint32_t G, const Draw& draw) {
    if (!nb.fast) return -1;
    const int tn = s.tab_n;
    const int dl = nb.dl, dg = nb.dg;
    float sabs = nb.sabs;
    float vol = 0.f, itf = 0.f;
    float sterm = 0.f;
    // one term difference table[x1] - table[x0] as a leaf
    auto leaf = [&](const float* hi, const float* lo, int64_t x1, int64_t x0) -> float {
        const float a = hi[x1], b = hi[x0];
        const float r = (a - b) + (lo[x1] - lo[x0]);
        sabs += fabsf(r);
        sterm += fabsf(a) + fabsf(b);
        return r;
    };
    if (L) {
        const int ty = li - 1;
        const int64_t v = volume[L], i = interface[L];
        if (v >= 1 && v < tn && i + dl >= 0 && i + dl < tn && i < tn) {
            vol += leaf(s.vterm32 + ty * tn, s.vterm32lo + ty * tn, v - 1, v);
            itf += leaf(s.iterm32 + ty * tn, s.iterm32lo + ty * tn, i + dl, i);
        } else {
            return -1;
        }
    }
    if (G) {
        const int ty = gi - 1;
        const int64_t v = volume[G], i = interface[G];
        if (v + 1 < tn && i + dg >= 0 && i + dg < tn && i < tn) {
            vol += leaf(s.vterm32 + ty * tn, s.vterm32lo + ty * tn, v + 1, v);
            itf += leaf(s.iterm32 + ty * tn, s.iterm32lo + ty * tn, i + dg, i);
        } else {
            return -1;
        }
    }
    if (!(sabs <= 1e30f && sterm <= 1e30f)) return -1;
    const float dh = (vol + itf) + nb.adh;
    const float eps = 4e-6f * sabs + 1e-12f * sterm + 1e-30f;
    const float hi = dh + eps, lo = dh - eps;
    if (hi <= 0.f) return 1;
    const uint32_t z = draw.z();
    if (lo > 64.f) {
        if (z != 0u) return 0;  // u >= 2^-32 > exp(-64)
    } else if (hi <= 64.f) {
        const float ulo = __uint2float_rd(z) * 2.3283064365386963e-10f;
        const float uhi = __fadd_ru(__uint2float_ru(z), 1.0f) * 2.3283064365386963e-10f;
        // u < exp(-hi) <= exp(-dh64) accepts whatever the sign of dh64
        const float elo = expf(-hi) * (1.0f - 3e-5f);
        if (uhi < elo) return 1;
        if (lo > 0.f) {
            const float ehi = expf(-lo) * (1.0f + 3e-5f);
            if (ulo > ehi) return 0;
        }
    }
    return -1;
}

// The exact decision: the reference's FP64 operation order (counted).
template <int NE, class SigT, class Draw>
__device__ __noinline__ bool decide_exact(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                          const uint32_t* volume, const uint32_t* interface, int64_t t, uint32_t L,
                                          uint32_t G, const Draw& draw) {
    if (s.stats) atomicAdd(&s.stats[CPM_STAT_EXACT_DECISIONS], 1ull);
    const DeltaOut o = delta_h<NE, SigT>(s, sig, adh_of, volume, interface, t, L, G);
    return metropolis(o.dh, o.dh > 0.0 ? draw.u() : 0.0);
}

template <int NE, class SigT, class Draw>
__device__ __forceinline__ bool decide_move(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                            const uint32_t* volume, const uint32_t* interface, int64_t t, uint32_t L,
                                            uint32_t G, const Draw& draw, int& dl, int& dg) {
    const NeighbourPart nb = decide_neighbours<NE, SigT, int64_t>(s, sig, adh_of, s.energy_off, t, L, G);
    dl = nb.dl;
    dg = nb.dg;
    const int r = decide_cells(s, nb, adh_of[L], adh_of[G], volume, interface, L, G, draw);
    if (r >= 0) return r != 0;
    return decide_exact<NE, SigT, Draw>(s, sig, adh_of, volume, interface, t, L, G, draw);
}

// ------------------------------------------------------ modes of the loop ----
// Acceptance by Metropolis-Hastings and the Act term, on a whole padded
// lattice (the global sweep, the shared-memory resident sweep and the
// parity harness; the tiled sweep restates the Act term's geometric means
// on its box, TileProc::act_gm). Both decide in FP64 with the reference's
// operation order; pow and exp are CUDA's, within an ulp of the host
// library's. The acquisition MCS lives in HBM.

// Interior padded index a (possibly halo) padded index stands for under a
// periodic boundary (energy.rs:363-376 canonical_flat); itself otherwise.
__device__ __forceinline__ int64_t act_canonical(const SimDesc& s, int64_t f) {
    if (!s.periodic) return f;
    int64_t r = f, out = 0;
    for (int d = 0; d < 3; ++d) {
        if (d >= s.D) break;
        int64_t c = r / s.strides[d];
        r -= c * s.strides[d];
        if (c == 0) c = s.dims[d];
        else if (c == s.pdims[d] - 1) c = 1;
        out += c * s.strides[d];
    }
    return out;
}

// product^(1/count), the geometric mean's last step (energy.rs:410), without
// the FP64 pow where its value is exact: a zero product (a retained site
// with no activity left, the usual case once Max_Act MCS have passed) gives
// +0, and one retained site gives the product itself, both as a correctly
// rounded pow (the host library's) returns them.
__device__ __forceinline__ double act_root(double product, uint32_t count) {
    if (product == 0.0) return 0.0;
    if (count == 1u) return product;
    return pow(product, __ddiv_rn(1.0, (double)count));
}

// Geometric mean of the activity max(0, max_act - (mcs - birth)) over
// `site` and its copy neighbours owned by `relevant` (energy.rs:377-412).
template <class SigT>
__device__ __forceinline__ double act_geometric_mean(const SimDesc& s, const SigT* sig, int64_t site,
                                                     uint32_t relevant, uint32_t max_act, uint64_t mcs) {
    const int64_t is = act_canonical(s, site);
    double product = 1.0;
    uint32_t count = 0;
    for (int k = -1; k < s.n_copy; ++k) {
        const int64_t c = k < 0 ? is : act_canonical(s, is + s.copy_off[k]);
        if ((uint32_t)sig[c] != relevant) continue;
        const uint64_t b = s.birth[c];
        const uint64_t elapsed = mcs > b ? mcs - b : 0ull;
        const uint64_t a = (uint64_t)max_act > elapsed ? (uint64_t)max_act - elapsed : 0ull;
        if (a == 0) return 0.0;  // the product stays zero whatever follows (every factor is finite)
        product = __dmul_rn(product, (double)a);
        count += 1;
    }
    return act_root(product, count);
}

// energy.rs:441-451: -(lambda_act / max_act) (GM_src - GM_tgt) of the
// gaining cell's type; 0 when the medium gains.
template <class SigT>
__device__ __forceinline__ double act_delta(const SimDesc& s, const SigT* sig, const uint16_t* adh_of, int64_t t,
                                            int64_t src, uint32_t L, uint32_t G, uint64_t mcs) {
    if (G == 0) return 0.0;
    const int ty = adh_of[G] - 1;
    const double lambda = s.lambda_act[ty];
    const uint32_t mx = s.max_act[ty];
    const double gs = act_geometric_mean(s, sig, src, G, mx, mcs);
    const double gt = act_geometric_mean(s, sig, t, L, mx, mcs);
    return __dmul_rn(-__ddiv_rn(lambda, (double)mx), __dsub_rn(gs, gt));
}

// monte_carlo.rs:147-196 for a total delta-H `dh`: Metropolis, or
// Metropolis-Hastings with the copy-neighbour counts n_A (losing) and n_B
// (gaining) of the target (rejected outright when n_A = 0).
template <class SigT, class Draw>
__device__ __forceinline__ bool accept_modes(const SimDesc& s, const SigT* sig, int64_t t, uint32_t L, uint32_t G,
                                             double dh, const Draw& draw) {
    if (s.acceptance == 0) return metropolis(dh, dh > 0.0 ? draw.u() : 0.0);
    int na = 0, nb = 0;
    for (int k = 0; k < s.n_copy; ++k) {
        const uint32_t c = (uint32_t)sig[t + s.copy_off[k]];
        na += c == L;
        nb += c == G;
    }
    if (na == 0) return false;
    // dh <= 0 and na >= nb: both factors round to >= 1, so min(ratio, 1) = 1 > u
    if (dh <= 0.0 && na >= nb) return true;
    const double ratio = __dmul_rn(__ddiv_rn((double)na, (double)nb), exp(-dh));
    return draw.u() < fmin(ratio, 1.0);
}

// The sweeps' decision under Metropolis acceptance with the Act term: the
// Act delta first (exact FP64). When it is zero — both geometric means
// vanish, the usual case since one retained site past its Max_Act MCS
// zeroes a mean, or they are equal — the total dh + (+-0) decides as dh
// alone, which decide_move's float bracket and FP64 fallback decide
// exactly; otherwise the conservative part in FP64 plus the Act delta, in
// the reference's order. Metropolis-Hastings acceptance: decide_modes.
template <int NE, class SigT, class Draw>
__device__ __forceinline__ bool decide_modes_sweep(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                                   const uint32_t* volume, const uint32_t* interface, int64_t t,
                                                   int64_t src, uint32_t L, uint32_t G, uint64_t mcs,
                                                   const Draw& draw, int& dl, int& dg);

// The decision of one attempt under the configured modes; `dh_total`
// receives the delta-H the decision used (conservative + Act).
template <int NE, class SigT, class Draw>
__device__ __forceinline__ bool decide_modes(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                             const uint32_t* volume, const uint32_t* interface, int64_t t,
                                             int64_t src, uint32_t L, uint32_t G, uint64_t mcs, const Draw& draw,
                                             int& dl, int& dg, double& dh_total) {
    const DeltaOut o = delta_h<NE, SigT>(s, sig, adh_of, volume, interface, t, L, G);
    dl = o.dl;
    dg = o.dg;
    dh_total = s.act ? __dadd_rn(o.dh, act_delta(s, sig, adh_of, t, src, L, G, mcs)) : o.dh;
    return accept_modes(s, sig, t, L, G, dh_total, draw);
}

template <int NE, class SigT, class Draw>
__device__ __forceinline__ bool decide_modes_sweep(const SimDesc& s, const SigT* sig, const uint16_t* adh_of,
                                                   const uint32_t* volume, const uint32_t* interface, int64_t t,
                                                   int64_t src, uint32_t L, uint32_t G, uint64_t mcs,
                                                   const Draw& draw, int& dl, int& dg) {
    if (s.acceptance == 0 && s.act) {
        const double act = act_delta(s, sig, adh_of, t, src, L, G, mcs);
        if (act == 0.0) return decide_move<NE, SigT>(s, sig, adh_of, volume, interface, t, L, G, draw, dl, dg);
        const DeltaOut o = delta_h<NE, SigT>(s, sig, adh_of, volume, interface, t, L, G);
        dl = o.dl;
        dg = o.dg;
        return accept_modes(s, sig, t, L, G, __dadd_rn(o.dh, act), draw);
    }
    double dh_total = 0.0;
    return decide_modes<NE, SigT, Draw>(s, sig, adh_of, volume, interface, t, src, L, G, mcs, draw, dl, dg, dh_total);
}

// ------------------------------------------------------------- commit ----
// Nearest periodic image of `coord` to `centroid` (dynamics.rs:187-202).
__device__ __forceinline__ int64_t nearest_image(int64_t coord, double centroid, int64_t extent, bool periodic) {
    if (!periodic) return coord;
    int64_t best = coord;
    double bd = fabs(__dsub_rn((double)coord, centroid));
    const double d1 = fabs(__dsub_rn((double)(coord - extent), centroid));
    if (d1 < bd) { best = coord - extent; bd = d1; }
    const double d2 = fabs(__dsub_rn((double)(coord + extent), centroid));
    if (d2 < bd) { best = coord + extent; }
    return best;
}

// The same choice for centroid = fl(sum / vb), decided in integers:
// |p - r| < |q - r| for r = sum / vb  <=>  (p - q) (vb (p + q) - 2 sum) < 0.
// Where the exact distances differ they differ by at least 1/vb (opposite
// sides of r) or by L (same side), far above the FP64 rounding of the
// division and subtractions for |sum| < 2^40 and vb < 2^20; where they tie,
// r = (p + q) / 2 is a half-integer, so the FP64 centroid and distances are
// exact and compare equal too. Outside those ranges the FP64 form runs.
__device__ __forceinline__ int64_t nearest_image_exact(int64_t coord, int64_t sum, int64_t vb, int64_t extent,
                                                       bool periodic) {
    if (!periodic) return coord;
    const int64_t lim = (int64_t)1 << 40;
    if (sum >= lim || sum <= -lim || vb >= ((int64_t)1 << 20) || coord >= lim || coord <= -lim)
        return nearest_image(coord, (double)sum / (double)vb, extent, true);
    int64_t best = coord;
    // p = coord - L against q = coord: (p - q) = -L < 0
    if (vb * (2 * coord - extent) - 2 * sum > 0) best = coord - extent;
    // p = coord + L against the current best
    if (best == coord) {
        if (vb * (2 * coord + extent) - 2 * sum < 0) best = coord + extent;  // p - q = L > 0
    } else {
        if (vb * coord - sum < 0) best = coord + extent;                      // p - q = 2L > 0
    }
    return best;
}

// Writes sigma[t] = v and, under a periodic boundary, every halo cell that
// mirrors t (the local equivalent of lattice.rs:240-254's full refresh).
template <int D, class SigT>
__device__ __forceinline__ void write_site(const SimDesc& s, SigT* sig, const int* x, uint32_t v) {
    int alt[3][3], na[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) { na[d] = 1; alt[d][0] = 0; alt[d][1] = 0; alt[d][2] = 0; }
#pragma unroll
    for (int d = 0; d < D; ++d) {
        alt[d][0] = x[d] + 1;
        if (s.periodic) {
            if (x[d] == 0) alt[d][na[d]++] = s.pdims[d] - 1;       // far halo mirrors coordinate 0
            if (x[d] == s.dims[d] - 1) alt[d][na[d]++] = 0;        // near halo mirrors the last one
        }
    }
    for (int a = 0; a < na[0]; ++a)
        for (int b = 0; b < (D > 1 ? na[1] : 1); ++b)
            for (int c = 0; c < (D > 2 ? na[2] : 1); ++c) {
                int64_t f = (int64_t)alt[0][a] * s.strides[0];
                if (D > 1) f += (int64_t)alt[1][b] * s.strides[1];
                if (D > 2) f += (int64_t)alt[2][c] * s.strides[2];
                sig[f] = (SigT)v;
            }
}

// dynamics::commit for an accepted move whose cells this thread owns
// exclusively (contact is recounted at sample time, not maintained here).
template <int D, class SigT>
__device__ __forceinline__ void commit_move(const SimDesc& s, SigT* sig, uint32_t* volume, uint32_t* interface,
                                            int64_t* sum_pos, int64_t* sum_outer, const int* x, uint32_t L,
                                            uint32_t G, int dl, int dg) {
    write_site<D, SigT>(s, sig, x, G);
    if (L) {
        volume[L] -= 1;
        interface[L] += (uint32_t)dl;
        int64_t* sp = sum_pos + (int64_t)L * D;
        int64_t* so = sum_outer + (int64_t)L * D * D;
#pragma unroll
        for (int d = 0; d < D; ++d) sp[d] -= x[d];
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
            for (int e = 0; e < D; ++e) so[d * D + e] -= (int64_t)x[d] * x[e];
    }
    if (G) {
        const uint32_t vnew = volume[G] + 1;
        volume[G] = vnew;
        interface[G] += (uint32_t)dg;
        uint32_t vb = vnew >= 1 ? vnew - 1 : 0;
        if (vb < 1) vb = 1;
        int64_t* sp = sum_pos + (int64_t)G * D;
        int64_t* so = sum_outer + (int64_t)G * D * D;
        int64_t img[3];
#pragma unroll
        for (int d = 0; d < D; ++d) img[d] = nearest_image_exact(x[d], sp[d], vb, s.dims[d], s.periodic != 0);
#pragma unroll
        for (int d = 0; d < D; ++d) sp[d] += img[d];
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
            for (int e = 0; e < D; ++e) so[d * D + e] += img[d] * img[e];
    }
}

// Interior coordinates of a padded flat index.
template <int D>
__device__ __forceinline__ void coords_of(const SimDesc& s, int64_t f, int* x) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const int64_t c = f / s.strides[d];
        f -= c * s.strides[d];
        x[d] = (int)c - 1;
    }
}

}  // namespace cpmgpu
