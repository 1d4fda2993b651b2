// Tiled sweep for lattices too large for one CTA's shared memory (the
// kernel source of cpm_tiled.cu and cpm_tiled_odd.cu).
//
// Every MCS the lattice is cut into an even number of tiles per axis, at a
// random offset (periodic lattices), and the tiles are coloured by the
// parity of their tile coordinates (4 colours in 2D, 8 in 3D). A sub-phase
// processes all tiles of one colour at once, one CTA per tile: same-colour
// tiles are a whole tile apart, so no attempt in one reads a site another
// writes. A cell that reaches into two tiles of the same colour would couple
// them through its volume and interface; each sub-phase therefore starts
// with a claim step: every active tile registers the cells of its box with
// a 64-bit atomicMin of (sub-phase epoch, tile id), a grid barrier follows,
// and a tile only changes cells it owns (the lowest claiming tile). Moves
// that involve a cell owned by another tile are counted and skipped (for
// compact cells this needs a cell wider than a tile, ~21 sites).
//
// Inside its tile a CTA stages the box (tile + 1-site rim) into shared
// memory, runs the site-colour passes of the tile in random order, and
// resolves each pass exactly as the resident sweep does (speculative FP64
// evaluation, then the fixpoint that finalises rejection chains, then
// parallel commits of cell-disjoint accepts). It then writes the tile's
// sites (plus their periodic halo mirrors), the owned cells' V/I and
// nothing else back to HBM; the position sums are updated in place with
// L2-coherent accesses.
//
// All CTAs are co-resident (cooperative launch); the grid barrier is a
// counter/generation pair with a bounded spin that records a timeout and
// returns instead of hanging.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <type_traits>

#include "cpm_common.h"
#include "cpm_device.cuh"
#include "cpm_kernels.h"

// The unit that compiles the even-sided Metropolis kernels also compiles the
// host entry points the four kernel units share.
#if !defined(CPM_TILED_ODD_UNIT) && !defined(CPM_TILED_MODES_UNIT)
#define CPM_TILED_MAIN_UNIT
#endif

namespace cpmgpu {

constexpr int TB = 256;          // threads per CTA
constexpr int TCMAX = 1024;      // candidate slots per tile pass
constexpr int TMAX_BOX = 48 * 48 * 48;  // largest shared box (sites)
constexpr int TCHG = 1024;       // changed sites listed per sub-phase (beyond: the whole tile is written back)
enum : uint32_t {
    T_ACC = 1u << 3, T_PEND = 1u << 4, T_FIN = 1u << 5, T_GUARD = 1u << 6, T_DONE = 1u << 7,
};
enum : uint32_t { TAG_TILE = 3u };

struct TileGrid {
    int nt[3];        // tiles per axis (even)
    int off[3];       // tiling offset per axis (periodic) or 0
    int colors;       // 2^D
};

// Tile j on an axis covers global coordinates [off + b_j, off + b_{j+1}) mod L,
// b_j = floor(j * L / nt).
__device__ __forceinline__ int tile_begin(int j, int L, int nt) { return (int)(((unsigned)j * (unsigned)L) / (unsigned)nt); }

struct BarrierState {
    unsigned int count;
    unsigned int gen;
    int error;
    int pad;
};

__device__ __forceinline__ void red_release_add(unsigned int* p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier: one release-add per CTA on a counter that only grows
// within a launch (the host zeroes it), and acquire loads until it reaches
// `epoch` * n. The wait gives up after 2 s of wall time, records the
// timeout and returns false instead of hanging.
static __device__ bool grid_sync(BarrierState* b, unsigned int n, unsigned int& epoch) {
    __shared__ int s_ok;
    ++epoch;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int target = epoch * n;
        red_release_add(&b->count, 1u);
        int ok = 1;
        if (ld_acquire(&b->count) < target) {
            const unsigned long long t0 = global_ns();
            unsigned int spins = 0;
            while (ld_acquire(&b->count) < target) {
                __nanosleep(20);
                if ((++spins & 255u) == 0u &&
                    (global_ns() - t0 > 2000000000ull || *((volatile int*)&b->error))) {
                    ok = 0;
                    break;
                }
            }
        }
        if (!ok) atomicExch(&b->error, 1);
        s_ok = ok && !*((volatile int*)&b->error);
    }
    __syncthreads();
    return s_ok != 0;
}

// Per-thread event counts (32-bit: a launch covers at most 2^18 MCS) and,
// in shared memory, the cycle counters thread 0 (lane 0 in the warp
// resolution) keeps for the profile (CPM_STAT_CYC_*).
enum TileCyc { TC_PASS = 0, TC_STAGE, TC_SYNC, TC_BUILD, TC_EVAL, TC_FIX, TC_APPLY, TC_LOWER, TC_CLAIM, TC_BAR1,
               TC_BAR2, TC_N };
struct TileCounters {
    uint32_t nonnull, topo, guard, evaluated, accepted, rounds, deferred, wide;
    unsigned long long* cyc;  // TC_N shared counters
    __device__ __forceinline__ void tick(int which, long long d) {
        if (threadIdx.x == 0) cyc[which] += (unsigned long long)d;
    }
};

// The attempt's draw with its top word taken from the per-site table staged
// with the box; the full 53-bit u (FP64 fallback only) is recomputed.
struct TileDraw {
    uint64_t seed, mcs;
    uint32_t site, zv;
    __device__ double u() const { return u53(site_draw(seed, mcs, site)); }
    __device__ uint32_t z() const { return zv; }
};

// preserves_topology on the box with 32-bit local offsets
template <int D>
__device__ __forceinline__ bool tile_simple(const uint16_t* sig, const int* toff, int t, uint32_t losing,
                                            const uint32_t* t2, const uint64_t* t3) {
    if (losing == 0) return true;  // medium is exempt (connectivity.rs:48-50)
    constexpr int NF = D == 2 ? 8 : 26;
    uint32_t p = 0;
#pragma unroll
    for (int i = 0; i < NF; ++i) p |= (uint32_t)((uint32_t)sig[t + toff[i]] == losing) << i;
    return D == 2 ? table2d_bit(t2, p) : table3d_bit(t3, p);
}

// MODES: the simulation uses Metropolis-Hastings acceptance or the Act term
// (compiled as separate kernels, so that the Metropolis kernels keep their
// registers).
template <int D, int NE, bool MODES>
struct TileProc {
    const SimDesc& g;     // global descriptor
    SimDesc& l;           // box descriptor: local strides/offsets, same parameters
    uint16_t* sig;        // box sigma
    int* gx0;             // global interior coordinate of box position 1 on each axis
    uint32_t *vol, *itf, *b0, *b1;
    uint16_t* adh;
    uint8_t *dirty, *own, *mod;
    // candidate arrays of the pass being resolved (a slice of the tile's
    // candidate storage: see at())
    uint32_t *c_site, *c_key, *c_cells, *c_flags, *c_gf, *c_z;
    int16_t* c_dl;
    // the neighbour half of each candidate's decision (decide_neighbours,
    // computed while building the pass) and its global coordinates
    float *c_adh, *c_sabs;
    uint32_t* c_xy;   // axis 0 | axis 1 << 16
    uint16_t* c_x2;   // axis 2 (3D)
    // sites whose sigma a commit changed in this sub-phase (box indices)
    uint32_t* chg;
    int* s_nchg;
    const uint64_t* t3;
    int* s_n;
    // the candidate storage's base pointers; at(off) points the candidate
    // arrays at the slice starting at candidate `off`
    uint32_t *b_site, *b_key, *b_cells, *b_flags, *b_gf, *b_z, *b_xy;
    int16_t* b_dl;
    float *b_adh, *b_sabs;
    uint16_t* b_x2;
    __device__ __forceinline__ void at(int off) {
        c_site = b_site + off; c_key = b_key + off; c_cells = b_cells + off; c_flags = b_flags + off;
        c_gf = b_gf + off; c_z = b_z + off; c_xy = b_xy + off; c_dl = b_dl + off; c_adh = b_adh + off;
        c_sabs = b_sabs + off; c_x2 = b_x2 + off;
    }
    // The box holds box-local cell slots, not cell ids: slot s >= 1 is
    // the cell clist[s - 1], slot 0 the medium; every per-cell array is
    // indexed by slot. Position sums of the first cl_cap slots are staged in
    // shared memory, the others live in HBM (through L2).
    const uint32_t* clist;
    long long *ssp, *sso;
    int cl_cap;
    const int* bdims;  // box extent per axis (tile + rim)
    uint64_t mcs;      // the MCS being swept (acquisition MCS of the Act term)

    __device__ __forceinline__ bool sums_of(uint32_t s, long long*& sp, long long*& so) const {
        const int k = (int)s - 1;
        if (k < cl_cap) {
            sp = ssp + (long long)k * D;
            so = sso + (long long)k * D * D;
            return true;
        }
        const uint32_t id = clist[k];
        sp = (long long*)g.sum_pos + (long long)id * D;
        so = (long long*)g.sum_outer + (long long)id * D * D;
        return false;
    }
    static __device__ __forceinline__ long long ld_sum(const long long* p, bool shared) { return shared ? *p : __ldcg(p); }
    static __device__ __forceinline__ void st_sum(long long* p, long long v, bool shared) {
        if (shared) *p = v;
        else __stcg(p, v);
    }

    __device__ int gcoord(int d, int local) const {  // box position -> global interior coordinate
        int x = gx0[d] + local - 1;
        const int L = g.dims[d];
        if (g.periodic) { x %= L; if (x < 0) x += L; }
        return x;
    }
    __device__ int gflat_of_box(int lt, int* xg) const {
        int f = 0, r = lt;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int q = r / (int)l.strides[d];
            r -= q * (int)l.strides[d];
            xg[d] = gcoord(d, q);
            f += (xg[d] + 1) * (int)g.strides[d];
        }
        return f;
    }

    // ---- Metropolis-Hastings acceptance and the Act term (MODES kernels)
    // The whole decision in FP64 with the reference's operation order, as
    // decide_modes makes it on a whole lattice. The box holds the target's
    // copy neighbourhood; the Act term also reads the source's, which can
    // leave the box by one site. Such a site lies in a neighbouring tile of
    // another colour (tiles are at least 8 sites wide), which no CTA changes
    // during this sub-phase, so it is read from the lattice in HBM. The
    // acquisition MCS of every site lives in HBM; a commit writes it for the
    // site it changes (L2 accesses: written and read by other CTAs in later
    // sub-phases).

    // Geometric mean of the activity max(0, max_act - (mcs - birth)) over
    // box position q and its copy neighbours owned by slot `rel`
    // (energy.rs:377-412), in the reference's order: q, then the copy
    // offsets in stencil order.
    __device__ double act_gm(int q, uint32_t rel, uint32_t max_act, uint64_t m) const {
        int x[3] = {0, 0, 0};
        {
            int r = q;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                x[d] = r / (int)l.strides[d];
                r -= x[d] * (int)l.strides[d];
            }
        }
        const uint32_t rel_id = rel ? clist[rel - 1] : 0u;
        double product = 1.0;
        uint32_t count = 0;
        for (int k = -1; k < g.n_copy; ++k) {
            int y[3] = {x[0], x[1], x[2]};
            bool in_box = true;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                if (k >= 0) y[d] += g.copy_vec[k][d];
                in_box &= y[d] >= 0 && y[d] < bdims[d];
            }
            int gf = 0;
            if (in_box) {
                int qq = 0;
#pragma unroll
                for (int d = 0; d < D; ++d) qq += y[d] * (int)l.strides[d];
                if ((uint32_t)sig[qq] != rel) continue;
                int xg[3];
                gf = gflat_of_box(qq, xg);  // the interior site (periodic) or the fixed halo site
            } else {
                bool outside = false, padded = true;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const int xx = gcoord(d, y[d]);
                    outside |= xx < 0 || xx >= g.dims[d];      // a fixed lattice's medium halo
                    padded &= xx >= -1 && xx <= g.dims[d];   // within the padded lattice
                    gf += (xx + 1) * (int)g.strides[d];
                }
                const uint32_t id = outside ? 0u : __ldcg(g.sigma + gf);
                if (id != rel_id || !padded) continue;
            }
            const uint64_t b = __ldcg(g.birth + gf);
            const uint64_t elapsed = m > b ? m - b : 0ull;
            const uint64_t a = (uint64_t)max_act > elapsed ? (uint64_t)max_act - elapsed : 0ull;
            if (a == 0) return 0.0;  // the product stays zero whatever follows
            product = __dmul_rn(product, (double)a);
            count += 1;
        }
        return act_root(product, count);
    }

    // energy.rs:441-451 on the box: -(lambda_act / max_act) (GM_src - GM_tgt)
    // of the gaining cell's type; 0 when the medium gains.
    __device__ double act_delta_box(int t, int src, uint32_t L, uint32_t G, uint64_t m) const {
        if (G == 0) return 0.0;
        const int ty = adh[G] - 1;
        const double lambda = g.lambda_act[ty];
        const uint32_t mx = g.max_act[ty];
        const double gs = act_gm(src, G, mx, m);
        const double gt = act_gm(t, L, mx, m);
        return __dmul_rn(-__ddiv_rn(lambda, (double)mx), __dsub_rn(gs, gt));
    }

    // decide_modes on the box: conservative delta-H (+ the Act term), then
    // Metropolis or Metropolis-Hastings (accept_modes counts the target's
    // copy neighbours, which the box holds).
    __device__ bool decide_box_modes(int t, int src, uint32_t L, uint32_t G, uint64_t m, const TileDraw& draw, int& dl,
                                     int& dg) const {
        const DeltaOut o = delta_h<NE, uint16_t>(l, sig, adh, vol, itf, t, L, G);
        dl = o.dl;
        dg = o.dg;
        const double dh = g.act ? __dadd_rn(o.dh, act_delta_box(t, src, L, G, m)) : o.dh;
        return accept_modes(l, sig, t, L, G, dh, draw);
    }

    // A MODES candidate's decision over its staged neighbour half, as
    // decide_modes_sweep makes it: under Metropolis acceptance the Act delta
    // first, and when it is zero the float bracket of the plain chain (the
    // total dh + (+-0) decides as dh); otherwise everything in FP64.
    __device__ bool decide_modes_staged(int t, int src, uint32_t L, uint32_t G, uint64_t m, const TileDraw& draw,
                                        const NeighbourPart& nb) const {
        if (g.acceptance == 0) {
            const double act = act_delta_box(t, src, L, G, m);
            if (act == 0.0) {
                int r = decide_cells(l, nb, adh[L], adh[G], vol, itf, L, G, draw);
                if (r < 0) r = decide_exact<NE, uint16_t>(l, sig, adh, vol, itf, t, L, G, draw) ? 1 : 0;
                return r != 0;
            }
            const DeltaOut o = delta_h<NE, uint16_t>(l, sig, adh, vol, itf, t, L, G);
            return accept_modes(l, sig, t, L, G, __dadd_rn(o.dh, act), draw);
        }
        int dl = 0, dg = 0;
        return decide_box_modes(t, src, L, G, m, draw, dl, dg);
    }

    // The candidate's decision on the current volumes and interfaces: the
    // cell half of decide_move over the neighbour half staged with the
    // candidate (sigma around it cannot change within its pass).
    __device__ void evaluate(int c, uint64_t mcs) {
        const uint32_t cells = c_cells[c];
        const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
        uint32_t fl = c_flags[c] & ~(T_ACC | T_GUARD);
        if (L != 0 && vol[L] <= l.min_cell_volume) {
            fl |= T_GUARD;
        } else {
            const int16_t dd = c_dl[c];
            NeighbourPart nb;
            nb.adh = c_adh[c];
            nb.sabs = c_sabs[c];
            nb.dl = (int)(int8_t)(dd & 0xFF);
            nb.dg = (int)(int8_t)((dd >> 8) & 0xFF);
            nb.fast = l.dj32 != nullptr;
            const TileDraw draw{g.seed, mcs, c_gf[c], c_z[c]};
            int r;
            if constexpr (MODES) {
                const int t = (int)c_site[c];
                r = decide_modes_staged(t, t + (int)l.copy_off[fl & 7u], L, G, mcs, draw, nb) ? 1 : 0;
            } else {
                r = decide_cells(l, nb, adh[L], adh[G], vol, itf, L, G, draw);
                if (r < 0) r = decide_exact<NE, uint16_t>(l, sig, adh, vol, itf, (int)c_site[c], L, G, draw) ? 1 : 0;
            }
            if (r) fl |= T_ACC;
        }
        c_flags[c] = fl;
    }

    // Commit in shared memory; position sums in HBM through L2. `mark` sets
    // the dirty bytes the block-wide resolve uses to find re-evaluations.
    __device__ void commit(int c, bool mark = true) {
        const int t = (int)c_site[c];
        const uint32_t cells = c_cells[c];
        const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
        const int16_t dd = c_dl[c];
        const int dl = (int)(int8_t)(dd & 0xFF), dg = (int)(int8_t)((dd >> 8) & 0xFF);
        int xg[3];
        const uint32_t xy = c_xy[c];
        xg[0] = (int)(xy & 0xFFFFu);
        xg[1] = (int)(xy >> 16);
        xg[2] = D > 2 ? (int)c_x2[c] : 0;
        sig[t] = (uint16_t)G;
        {
            const int k = atomicAdd(s_nchg, 1);
            if (k < TCHG) chg[k] = (uint32_t)t;
        }
        if constexpr (MODES) {
            if (g.act) __stcg(g.birth + c_gf[c], (uint32_t)mcs);  // energy.rs:453-458
        }
        if (L) {
            vol[L] -= 1;
            itf[L] += (uint32_t)dl;
            long long *sp, *so;
            const bool sh = sums_of(L, sp, so);
#pragma unroll
            for (int d = 0; d < D; ++d) st_sum(sp + d, ld_sum(sp + d, sh) - xg[d], sh);
#pragma unroll
            for (int d = 0; d < D; ++d)
#pragma unroll
                for (int e = 0; e < D; ++e)
                    st_sum(so + d * D + e, ld_sum(so + d * D + e, sh) - (long long)xg[d] * xg[e], sh);
            if (mark) dirty[L] = 1;
            mod[L] = 1;
        }
        if (G) {
            const uint32_t vnew = vol[G] + 1;
            vol[G] = vnew;
            itf[G] += (uint32_t)dg;
            uint32_t vb = vnew >= 1 ? vnew - 1 : 0;
            if (vb < 1) vb = 1;
            long long *sp, *so;
            const bool sh = sums_of(G, sp, so);
            long long img[3], cur[3];
#pragma unroll
            for (int d = 0; d < D; ++d) cur[d] = ld_sum(sp + d, sh);
#pragma unroll
            for (int d = 0; d < D; ++d) img[d] = nearest_image_exact(xg[d], cur[d], vb, g.dims[d], g.periodic != 0);
#pragma unroll
            for (int d = 0; d < D; ++d) st_sum(sp + d, cur[d] + img[d], sh);
#pragma unroll
            for (int d = 0; d < D; ++d)
#pragma unroll
                for (int e = 0; e < D; ++e) st_sum(so + d * D + e, ld_sum(so + d * D + e, sh) + img[d] * img[e], sh);
            if (mark) dirty[G] = 1;
            mod[G] = 1;
        }
    }

    // Resolution of a pass with n <= 32 candidates by one warp, candidate =
    // lane, with the same outcome as resolve(): `lower` holds the
    // lower-priority candidates that share a cell (the medium is not a
    // cell); a pending candidate is final once every lower pending one is a
    // final reject; final accepts are pairwise cell-disjoint and commit; a
    // pending candidate with a committed lower neighbour re-evaluates (a
    // committed candidate sharing a cell with a pending one always has the
    // lower key, or the pending one would have been a final reject).
    template <int K>
    using Mask = typename std::conditional<K == 1, uint32_t, uint64_t>::type;
    template <int K>
    __device__ __forceinline__ Mask<K> ballot_k(const bool (&p)[K]) const {
        Mask<K> m = __ballot_sync(0xffffffffu, p[0]);
        if (K > 1) m |= (Mask<K>)__ballot_sync(0xffffffffu, p[K > 1 ? 1 : 0]) << (K > 1 ? 32 : 0);
        return m;
    }
    template <int K>
    __device__ __forceinline__ static Mask<K> bit_k(int c) { return (Mask<K>)1 << c; }

    // K = 1 handles n <= 32 candidates, K = 2 n <= 64 (candidate c = lane +
    // 32 q, bit c of the 64-bit masks).
    //
    // The build has already made every candidate's first decision.
    template <int K>
    __device__ void resolve_warp(int n, uint64_t mcs, TileCounters& ct) {
        const int lane = threadIdx.x & 31;
        long long t0 = clock64();
        long long tm = t0;
        uint32_t Lc[K], Gc[K], key[K], fl[K];
        Mask<K> lower[K];
        bool have[K];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const int c = lane + 32 * q;
            have[q] = c < n;
            const uint32_t cells = have[q] ? c_cells[c] : 0u;
            key[q] = have[q] ? c_key[c] : 0xFFFFFFFFu;
            Lc[q] = cells & 0xFFFFu;
            Gc[q] = cells >> 16;
        }
        // candidates sharing a cell: per-cell masks (b0: candidates 0..31,
        // b1: 32..63; both are free while the warp resolves), then keep the
        // sharers with a lower key
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (Lc[q]) { b0[Lc[q]] = 0u; if (K > 1) b1[Lc[q]] = 0u; }
            if (Gc[q]) { b0[Gc[q]] = 0u; if (K > 1) b1[Gc[q]] = 0u; }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < K; ++q) {
            uint32_t* bm = q == 0 ? b0 : b1;
            if (Lc[q]) atomicOr(&bm[Lc[q]], 1u << lane);
            if (Gc[q]) atomicOr(&bm[Gc[q]], 1u << lane);
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < K; ++q) {
            Mask<K> sh = 0;
            if (Lc[q]) sh |= (Mask<K>)b0[Lc[q]] | (K > 1 ? (Mask<K>)b1[Lc[q]] << (K > 1 ? 32 : 0) : (Mask<K>)0);
            if (Gc[q]) sh |= (Mask<K>)b0[Gc[q]] | (K > 1 ? (Mask<K>)b1[Gc[q]] << (K > 1 ? 32 : 0) : (Mask<K>)0);
            sh &= ~bit_k<K>(lane + 32 * q);
            Mask<K> lw = 0;
            while (sh) {
                const int j = K == 1 ? __ffs((uint32_t)sh) - 1 : __ffsll((long long)sh) - 1;
                sh &= sh - 1;
                if (c_key[j] < key[q]) lw |= bit_k<K>(j);
            }
            lower[q] = lw;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < K; ++q) fl[q] = have[q] ? c_flags[lane + 32 * q] : 0u;
        Mask<K> pending = ballot_k<K>(have);
        long long t1 = clock64();
        ct.tick(TC_LOWER, t1 - tm);
        while (pending) {
            t0 = clock64();
            bool mine[K], rej[K];
#pragma unroll
            for (int q = 0; q < K; ++q) {
                mine[q] = (pending >> (lane + 32 * q)) & 1u;
                rej[q] = (fl[q] & T_GUARD) || !(fl[q] & T_ACC);
            }
            Mask<K> fin = 0;
            for (;;) {
                bool fr[K], nf[K];
#pragma unroll
                for (int q = 0; q < K; ++q) fr[q] = ((fin >> (lane + 32 * q)) & 1u) && rej[q];
                const Mask<K> frej = ballot_k<K>(fr);
#pragma unroll
                for (int q = 0; q < K; ++q) nf[q] = mine[q] && (lower[q] & pending & ~frej) == 0;
                const Mask<K> f2 = ballot_k<K>(nf);
                if (f2 == fin) break;
                fin = f2;
            }
            t1 = clock64();
            ct.tick(TC_FIX, t1 - t0);
            bool cm[K];
#pragma unroll
            for (int q = 0; q < K; ++q) {
                const bool is_fin = (fin >> (lane + 32 * q)) & 1u;
                cm[q] = is_fin && !rej[q];
                if (is_fin) {
                    if (fl[q] & T_GUARD) ct.guard++;
                    else ct.evaluated++;
                }
                if (cm[q]) {
                    commit(lane + 32 * q, false);
                    ct.accepted++;
                }
            }
            const Mask<K> committed = ballot_k<K>(cm);
            pending &= ~fin;
            ct.rounds++;
            __syncwarp();
#pragma unroll
            for (int q = 0; q < K; ++q) {
                const int c = lane + 32 * q;
                if (((pending >> c) & 1u) && (lower[q] & committed)) {
                    evaluate(c, mcs);
                    fl[q] = c_flags[c];
                }
            }
            __syncwarp();
            ct.tick(TC_APPLY, clock64() - t1);
        }
    }

    // The block-wide resolution (more than 64 candidates); the build has
    // made the first decisions.
    __device__ void resolve(int n, uint64_t mcs, TileCounters& ct) {
        const int tid = threadIdx.x;
        long long t0 = clock64();
        long long t1 = t0;
        for (;;) {
            t0 = clock64();
            // finality as in the resident sweep: final unless an accepting
            // candidate lies in the lower closure (per-cell minimum key of
            // accepting or tainted candidates, propagated across cells)
            for (int c = tid; c < n; c += TB) {
                if (!(c_flags[c] & T_PEND)) continue;
                const uint32_t cells = c_cells[c];
                if (cells & 0xFFFFu) b0[cells & 0xFFFFu] = 0xFFFFFFFFu;
                if (cells >> 16) b0[cells >> 16] = 0xFFFFFFFFu;
            }
            __syncthreads();
            for (int c = tid; c < n; c += TB) {
                const uint32_t fl = c_flags[c];
                if (!(fl & T_PEND) || !(fl & T_ACC) || (fl & T_GUARD)) continue;
                const uint32_t cells = c_cells[c], key = c_key[c];
                if (cells & 0xFFFFu) atomicMin(&b0[cells & 0xFFFFu], key);
                if (cells >> 16) atomicMin(&b0[cells >> 16], key);
            }
            for (;;) {
                __syncthreads();
                int changed = 0;
                for (int c = tid; c < n; c += TB) {
                    if (!(c_flags[c] & T_PEND)) continue;
                    const uint32_t cells = c_cells[c], key = c_key[c];
                    const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
                    if (!((L && key > b0[L]) || (G && key > b0[G]))) continue;
                    if (L && atomicMin(&b0[L], key) > key) changed = 1;
                    if (G && atomicMin(&b0[G], key) > key) changed = 1;
                }
                if (!__syncthreads_or(changed)) break;
            }
            t1 = clock64();
            ct.tick(TC_FIX, t1 - t0);
            int left = 0;
            for (int c = tid; c < n; c += TB) {
                uint32_t fl = c_flags[c];
                if (!(fl & T_PEND)) continue;
                const uint32_t cells = c_cells[c], key = c_key[c];
                const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
                if ((L && key > b0[L]) || (G && key > b0[G])) { left = 1; continue; }
                fl &= ~T_PEND;
                if (fl & T_GUARD) ct.guard++;
                else {
                    ct.evaluated++;
                    if (fl & T_ACC) { commit(c); fl |= T_DONE; ct.accepted++; }
                }
                c_flags[c] = fl;
            }
            ct.rounds++;
            const int more = __syncthreads_or(left);
            ct.tick(TC_APPLY, clock64() - t1);
            if (!more) break;
            t1 = clock64();
            for (int c = tid; c < n; c += TB) {
                if (!(c_flags[c] & T_PEND)) continue;
                const uint32_t cells = c_cells[c];
                if (dirty[cells & 0xFFFFu] || dirty[cells >> 16]) evaluate(c, mcs);
            }
            __syncthreads();
            for (int c = tid; c < n; c += TB) {
                const uint32_t fl = c_flags[c];
                if (!(fl & T_DONE)) continue;
                const uint32_t cells = c_cells[c];
                dirty[cells & 0xFFFFu] = 0;
                dirty[cells >> 16] = 0;
                c_flags[c] = fl & ~T_DONE;
            }
            __syncthreads();
            ct.tick(TC_APPLY, clock64() - t1);
        }
        for (int c = tid; c < n; c += TB) {
            if (!(c_flags[c] & T_DONE)) continue;
            const uint32_t cells = c_cells[c];
            dirty[cells & 0xFFFFu] = 0;
            dirty[cells >> 16] = 0;
        }
        __syncthreads();
    }
};

struct TileShared {
    uint32_t sig, sid, vol, itf, b0, b1, adh, dirty, own, mod, clist, ssp, sso, rseen, rslot, chg, pass, c_site,
        c_key, c_cells, c_flags, c_gf, c_z, c_dl, c_adh, c_sabs, c_xy, c_x2, total;
};

__host__ __device__ inline uint32_t tl_take(uint32_t& off, uint64_t b) {
    const uint32_t o = off;
    off = (uint32_t)((off + b + 15) & ~(uint64_t)15);
    return o;
}
// reg_smem: the cell registry (a stamp and a slot per cell id) is kept in
// shared memory too (else in HBM, for lattices with many cells).
__host__ __device__ inline TileShared tile_shared(int box_sites, int n_cells, int cl_cap, int D, bool reg_smem) {
    TileShared s;
    uint32_t off = 0;
    // slots: the medium and at most one per box site (or per cell)
    const uint64_t n1 = (uint64_t)(box_sites < n_cells ? box_sites : n_cells) + 1;
    s.sig = tl_take(off, (uint64_t)box_sites * 2);
    s.vol = tl_take(off, n1 * 4);
    s.itf = tl_take(off, n1 * 4);
    s.b0 = tl_take(off, n1 * 4);
    s.b1 = tl_take(off, n1 * 4);
    s.adh = tl_take(off, n1 * 2);
    s.dirty = tl_take(off, n1);
    s.own = tl_take(off, n1);
    s.mod = tl_take(off, n1);
    s.clist = tl_take(off, n1 * 4);
    s.ssp = tl_take(off, (uint64_t)cl_cap * D * 8);
    s.sso = tl_take(off, (uint64_t)cl_cap * D * D * 8);
    s.rseen = tl_take(off, reg_smem ? ((uint64_t)n_cells + 1) * 4 : 0);
    s.rslot = tl_take(off, reg_smem ? ((uint64_t)n_cells + 1) * 2 : 0);
    s.chg = tl_take(off, TCHG * 4);
    s.pass = tl_take(off, (27 * 12 + 27 + 28 + 27 * 6) * 4);  // per-pass geometry and counters
    s.c_site = tl_take(off, TCMAX * 4);
    s.c_key = tl_take(off, TCMAX * 4);
    s.c_cells = tl_take(off, TCMAX * 4);
    s.c_flags = tl_take(off, TCMAX * 4);
    s.c_gf = tl_take(off, TCMAX * 4);
    s.c_z = tl_take(off, TCMAX * 4);
    s.c_adh = tl_take(off, TCMAX * 4);
    s.c_sabs = tl_take(off, TCMAX * 4);
    s.c_xy = tl_take(off, TCMAX * 4);
    s.c_dl = tl_take(off, TCMAX * 2);
    s.c_x2 = tl_take(off, TCMAX * 2);
    // the staged cell ids, before they become slots: only used while a box
    // is staged, so they share the candidate arrays when they fit there
    s.sid = (uint64_t)box_sites * 4 <= (uint64_t)(s.c_x2 + TCMAX * 2 - s.c_site) ? s.c_site
                                                                                   : tl_take(off, (uint64_t)box_sites * 4);
    s.total = off;
    return s;
}

// Shared-memory copy of the float energy tables (J, adhesion differences,
// term tables and their remainders): (n+1)^2 + (n+1)^3 + 4 n tab_n floats.
#ifdef CPM_TILED_MAIN_UNIT
size_t tiled_table_bytes(int n_types, int tab_n) {
    const size_t n1 = (size_t)n_types + 1;
    return (n1 * n1 + n1 * n1 * n1 + 4 * (size_t)n_types * (size_t)tab_n) * 4;
}
#endif

// ODD: the lattice has an odd periodic side, whose last coordinate takes a
// third site colour (compiled separately, so that the even-sided kernels
// keep their two-colour index arithmetic).
template <int D, int NE, bool ODD, bool MODES>
__global__ void __launch_bounds__(TB, 1) tiled_kernel(SimDesc* simp, uint64_t n_mcs, TileGrid tg_in, BarrierState* bar,
                                                   unsigned long long* claims, const uint64_t* t3, int max_box,
                                                   int tables_in_smem, int barrier_extra, int cl_cap,
                                                   int reg_smem, uint32_t* seen_all, uint32_t* slot_all) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ SimDesc gsd, lsd;
    __shared__ int s_n, s_tile, s_ncell, s_box_dims[3], s_gx0[3], s_g0[3], s_tcnt[3];
    __shared__ int perm[8], sperm[27];
    __shared__ uint32_t s_pkey[27], s_swap[27];
    __shared__ int s_nchg;
    // the box's stencils as 32-bit local index offsets
    __shared__ int s_eoff[CPM_MAX_STENCIL], s_toff[CPM_MAX_STENCIL], s_coff[6];
    __shared__ int s_ncls[3];
    __shared__ unsigned long long sstat[8];
    const int tid = threadIdx.x;
    if (tid == 0) gsd = *simp;
    if (tid < 8) sstat[tid] = 0;
    __syncthreads();
    // site colours per axis: the two parities, plus (ODD) the last
    // coordinate of an odd periodic axis as a third
    if (tid < 3) s_ncls[tid] = tid < D ? ((ODD && gsd.periodic && (gsd.dims[tid] & 1)) ? 3 : 2) : 1;
    __syncthreads();
    const int n_cls = ODD ? s_ncls[0] * s_ncls[1] * s_ncls[2] : 1 << D;
    if (tables_in_smem && gsd.dj32 != nullptr) {
        // the float energy tables move next to the tile state (no global
        // loads in the common-case decision)
        float* tb = (float*)(sm + tile_shared(max_box, gsd.n_cells, cl_cap, D, reg_smem != 0).total);
        const int n1 = gsd.n_types + 1, nj = n1 * n1, nd = n1 * n1 * n1, nv = gsd.n_types * gsd.tab_n;
        for (int q = tid; q < nj; q += TB) tb[q] = gsd.J32[q];
        for (int q = tid; q < nd; q += TB) tb[nj + q] = gsd.dj32[q];
        for (int q = tid; q < nv; q += TB) {
            tb[nj + nd + q] = gsd.vterm32[q];
            tb[nj + nd + nv + q] = gsd.iterm32[q];
            tb[nj + nd + 2 * nv + q] = gsd.vterm32lo[q];
            tb[nj + nd + 3 * nv + q] = gsd.iterm32lo[q];
        }
        __syncthreads();
        if (tid == 0) {
            gsd.J32 = tb;
            gsd.dj32 = tb + nj;
            gsd.vterm32 = tb + nj + nd;
            gsd.iterm32 = tb + nj + nd + nv;
            gsd.vterm32lo = tb + nj + nd + 2 * nv;
            gsd.iterm32lo = tb + nj + nd + 3 * nv;
        }
        __syncthreads();
    }
    // the box descriptor: gsd's parameters, box geometry set per tile
    for (int q = tid; q < (int)(sizeof(SimDesc) / 8); q += TB) ((uint64_t*)&lsd)[q] = ((const uint64_t*)&gsd)[q];
    __syncthreads();
    const SimDesc& g = gsd;
    const int nblk = gridDim.x;
    const unsigned int arrivals = (unsigned int)(nblk + barrier_extra);  // barrier_extra: timeout test hook
    // This CTA's cell registry, per cell id: the stamp of the last tile that
    // listed the cell (unique within a launch: at most 2^18 MCS x 8
    // sub-phases x 1024 tiles per CTA; zeroed here) and its slot in that
    // tile's box. In shared memory when it fits (reg_smem), else in HBM
    // (n_cells + 1 words each per CTA).
    const TileShared ts0 = tile_shared(max_box, g.n_cells, cl_cap, D, reg_smem != 0);
    // per site-colour pass: class geometry (count, first, count before the
    // wrap, first past the wrap per axis), site count and prefix, and the
    // speculative build's candidate count, accept flag and event counts
    int(*s_pg)[12] = (int(*)[12])(sm + ts0.pass);
    int* s_pn = (int*)(sm + ts0.pass) + 27 * 12;
    int* s_pfx = s_pn + 27;
    int* s_pcnt = s_pfx + 28;
    int* s_pacc = s_pcnt + 27;
    int* s_pguard = s_pacc + 27;
    int* s_pnonnull = s_pguard + 27;
    int* s_ptopo = s_pnonnull + 27;
    int* s_pdef = s_ptopo + 27;
    uint32_t* seen_g = seen_all + (size_t)blockIdx.x * (size_t)(g.n_cells + 1);
    uint32_t* slot_g = slot_all + (size_t)blockIdx.x * (size_t)(g.n_cells + 1);
    for (int id = tid; id <= g.n_cells; id += TB) {
        if (reg_smem) ((uint32_t*)(sm + ts0.rseen))[id] = 0u;
        else seen_g[id] = 0u;
    }
    __syncthreads();
    // first listing of `id` under `stamp`; its slot; the slot recorded
    auto reg_first = [&](uint32_t id, uint32_t stamp) -> bool {
        if (reg_smem) return atomicExch((uint32_t*)(sm + ts0.rseen) + id, stamp) != stamp;
        return atomicExch(seen_g + id, stamp) != stamp;
    };
    auto reg_set = [&](uint32_t id, uint32_t sl) {
        if (reg_smem) ((uint16_t*)(sm + ts0.rslot))[id] = (uint16_t)sl;
        else slot_g[id] = sl;
    };
    auto reg_get = [&](uint32_t id) -> uint32_t {
        return reg_smem ? (uint32_t)((const uint16_t*)(sm + ts0.rslot))[id] : __ldcg(slot_g + id);
    };
    __shared__ unsigned long long s_cyc[TC_N];
    if (tid < TC_N) s_cyc[tid] = 0ull;
    __syncthreads();
    TileCounters ct = {0, 0, 0, 0, 0, 0, 0, 0, s_cyc};
    unsigned long long attempts = 0, tile_passes = 0;
    const uint64_t mcs0 = g.mcs;
    bool alive = true;
    unsigned int bar_epoch = 0;
    for (uint64_t m = 0; m < n_mcs && alive; ++m) {
        const uint64_t mcs = mcs0 + m;
        // ---- tiling of this MCS: random offset (periodic), random tile-colour order
        TileGrid tg = tg_in;
        {
            const uint4 r = aux_draw(g.seed, mcs, TAG_TILE, 0u, 0u);
            const uint32_t rr[3] = {r.x, r.y, r.z};
            for (int d = 0; d < D; ++d) tg.off[d] = g.periodic ? (int)(((unsigned long long)rr[d] * (unsigned)g.dims[d]) >> 32) : 0;
        }
        // Fisher-Yates over the tile colours; the draws first, one per thread
        if (tid > 0 && tid < tg.colors) {
            const uint4 r = aux_draw(g.seed, mcs, TAG_TILE, 1u, (uint32_t)tid);
            s_swap[tid] = (uint32_t)(((unsigned long long)r.x * (unsigned)(tid + 1)) >> 32);
        }
        __syncthreads();
        if (tid == 0) {
            for (int c = 0; c < tg.colors; ++c) perm[c] = c;
            for (int c = tg.colors - 1; c > 0; --c) {
                const int j = (int)s_swap[c];
                const int t = perm[c]; perm[c] = perm[j]; perm[j] = t;
            }
        }
        __syncthreads();
        int n_tiles = 1;
        for (int d = 0; d < D; ++d) n_tiles *= tg.nt[d];
        const int per_color = n_tiles / tg.colors;
        for (int ci = 0; ci < tg.colors && alive; ++ci) {
            const int color = perm[ci];
            const uint64_t epoch = mcs * 8 + (uint64_t)ci;
            const unsigned long long base_key = (unsigned long long)(0xFFFFFFFFull - (epoch & 0xFFFFFFFFull)) << 32;
            // tile k of this colour -> tile coordinates: colour bits are the parities
            auto tile_coords = [&](int k, int* tc) {
                int rem = k;
                for (int d = D - 1; d >= 0; --d) {
                    const int half = tg.nt[d] / 2;
                    const int q = rem % half;
                    rem /= half;
                    tc[d] = 2 * q + ((color >> d) & 1);
                }
            };
            const TileShared ts = tile_shared(max_box, g.n_cells, cl_cap, D, reg_smem != 0);
            auto stamp_of = [&](int k) -> uint32_t {
                return (uint32_t)((m * 8 + (uint64_t)ci) * 1024u + (uint32_t)(k / nblk)) + 1u;
            };
            uint32_t* clist = (uint32_t*)(sm + ts.clist);
            // box geometry of tile k: global origin, extents, local strides and offsets
            auto setup_tile = [&](int k) {
                int tc[3];
                tile_coords(k, tc);
                if (tid == 0) {
                    // lsd holds gsd's parameters since the kernel started;
                    // only the box geometry changes per tile
                    for (int d = 0; d < D; ++d) {
                        const int L = g.dims[d];
                        const int b0 = tile_begin(tc[d], L, tg.nt[d]), b1 = tile_begin(tc[d] + 1, L, tg.nt[d]);
                        s_gx0[d] = b0 + tg.off[d];
                        s_g0[d] = (b0 + tg.off[d]) % L;  // both terms are in [0, L)
                        s_tcnt[d] = b1 - b0;
                        s_box_dims[d] = b1 - b0 + 2;
                        lsd.dims[d] = b1 - b0;
                        lsd.pdims[d] = b1 - b0 + 2;
                    }
                    int64_t st = 1;
                    for (int d = D - 1; d >= 0; --d) { lsd.strides[d] = st; st *= lsd.pdims[d]; }
                    lsd.n_padded = st;
                    s_tile = k;
                    s_ncell = 0;
                }
                __syncthreads();
                // local stencil offsets from the integer offset vectors (one thread each)
                if (tid < CPM_MAX_STENCIL) {
                    const int kk = tid;
                    int64_t e = 0, t = 0, c = 0;
                    for (int d = 0; d < D; ++d) {
                        e += (int64_t)g.energy_vec[kk][d] * lsd.strides[d];
                        t += (int64_t)g.topo_vec[kk][d] * lsd.strides[d];
                        if (kk < 6) c += (int64_t)g.copy_vec[kk][d] * lsd.strides[d];
                    }
                    if (kk < g.n_energy) { lsd.energy_off[kk] = e; s_eoff[kk] = (int)e; }
                    lsd.topo_off[kk] = t;
                    s_toff[kk] = (int)t;
                    if (kk < g.n_copy) { lsd.copy_off[kk] = c; s_coff[kk] = (int)c; }
                }
                __syncthreads();
            };
            TileProc<D, NE, MODES> P{g, lsd, (uint16_t*)(sm + ts.sig), s_gx0, (uint32_t*)(sm + ts.vol),
                              (uint32_t*)(sm + ts.itf), (uint32_t*)(sm + ts.b0), (uint32_t*)(sm + ts.b1),
                              (uint16_t*)(sm + ts.adh), (uint8_t*)(sm + ts.dirty), (uint8_t*)(sm + ts.own),
                              (uint8_t*)(sm + ts.mod), (uint32_t*)(sm + ts.c_site), (uint32_t*)(sm + ts.c_key),
                              (uint32_t*)(sm + ts.c_cells), (uint32_t*)(sm + ts.c_flags), (uint32_t*)(sm + ts.c_gf),
                              (uint32_t*)(sm + ts.c_z), (int16_t*)(sm + ts.c_dl), (float*)(sm + ts.c_adh),
                              (float*)(sm + ts.c_sabs), (uint32_t*)(sm + ts.c_xy), (uint16_t*)(sm + ts.c_x2),
                              (uint32_t*)(sm + ts.chg), &s_nchg, t3, &s_n,
                              (uint32_t*)(sm + ts.c_site), (uint32_t*)(sm + ts.c_key), (uint32_t*)(sm + ts.c_cells),
                              (uint32_t*)(sm + ts.c_flags), (uint32_t*)(sm + ts.c_gf), (uint32_t*)(sm + ts.c_z),
                              (uint32_t*)(sm + ts.c_xy), (int16_t*)(sm + ts.c_dl), (float*)(sm + ts.c_adh),
                              (float*)(sm + ts.c_sabs), (uint16_t*)(sm + ts.c_x2),
                              clist, (long long*)(sm + ts.ssp), (long long*)(sm + ts.sso), cl_cap,
                              s_box_dims, mcs};
            uint32_t* sid = (uint32_t*)(sm + ts.sid);
            // Stage the box of the current tile: each distinct cell of the
            // box listed once (and claimed when `claim`) and given the next
            // slot, the box's sigma as slots, then the listed cells' V, I,
            // type and position sums by slot. Nothing writes sigma, V or I
            // between the two grid barriers of a sub-phase, so staging may
            // run before the claim barrier.
            auto stage_box = [&](int k, bool claim, uint32_t salt) {
                const unsigned long long key = base_key | (unsigned long long)k;
                const uint32_t stamp = stamp_of(k) + salt;
                int box = 1;
                for (int d = 0; d < D; ++d) box *= s_box_dims[d];
                // four sites per thread in flight: their sigma loads first, then the rest
                // the loop bound is uniform across the block: every lane reaches
                // the warp-wide match below, lanes past the box with id 0
                for (int base = 0; base < box; base += 4 * TB) {
                    const int q0 = base + tid;
                    int gfs[4];
                    uint32_t ids[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int q = q0 + u * TB;
                        int xg[3];
                        // a fixed lattice's rim outside the box maps to its medium halo
                        gfs[u] = q < box ? P.gflat_of_box(q, xg) : 0;
                        ids[u] = q < box ? __ldcg(g.sigma + gfs[u]) : 0u;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int q = q0 + u * TB;
                        const bool valid = q < box;
                        const uint32_t id = valid ? ids[u] : 0u;
                        // one lane per distinct id of the warp touches the cell's stamp
                        // (every lane takes part in the match; lanes past the box carry id 0)
                        const unsigned peers = __match_any_sync(0xffffffffu, id);
                        const bool leader = (int)(threadIdx.x & 31) == __ffs(peers) - 1;
                        if (!valid) continue;
                        sid[q] = id;
                        if (id && leader && reg_first(id, stamp)) {
                            if (claim) atomicMin(claims + id, key);
                            const int k1 = atomicAdd(&s_ncell, 1);
                            clist[k1] = id;
                            reg_set(id, (uint32_t)(k1 + 1));
                        }
                    }
                }
                // the tile's site-colour order and pass keys
                // (Fisher-Yates draws one per thread, then the swaps)
                if (tid > 0 && tid < n_cls) {
                    const uint4 rr = aux_draw(g.seed, mcs, TAG_TILE, 2u + (uint32_t)k, (uint32_t)tid);
                    s_swap[tid] = (uint32_t)(((unsigned long long)rr.x * (unsigned)(tid + 1)) >> 32);
                }
                if (tid < n_cls)
                    s_pkey[tid] = aux_draw(g.seed, mcs, TAG_PASS, (uint32_t)(tid * 64 + ci), (uint32_t)k).x;
                __syncthreads();  // every listing (and its slot write) is visible to the block
                if (tid == 0) {
                    for (int c = 0; c < n_cls; ++c) sperm[c] = c;
                    for (int c = n_cls - 1; c > 0; --c) {
                        const int j = (int)s_swap[c];
                        const int t = sperm[c]; sperm[c] = sperm[j]; sperm[j] = t;
                    }
                }
#pragma unroll 4
                for (int q = tid; q < box; q += TB) {
                    const uint32_t id = sid[q];
                    P.sig[q] = id ? (uint16_t)reg_get(id) : (uint16_t)0;
                }
                const int nc = s_ncell;
                for (int i = tid; i <= nc; i += TB) {
                    const uint32_t id = i < nc ? clist[i] : 0u;  // the medium rides along as slot 0
                    const int sl = i < nc ? i + 1 : 0;
                    P.vol[sl] = __ldcg(g.volume + id);
                    P.itf[sl] = __ldcg(g.interface + id);
                    P.adh[sl] = g.adh_of[id];
                    P.dirty[sl] = 0;
                    P.mod[sl] = 0;
                    if (i < nc && i < cl_cap) {
                        for (int d = 0; d < D; ++d) P.ssp[i * D + d] = __ldcg(g.sum_pos + (int64_t)id * D + d);
                        for (int d = 0; d < D * D; ++d) P.sso[i * D * D + d] = __ldcg(g.sum_outer + (int64_t)id * D * D + d);
                    }
                }
            };
            // own[slot]: the lowest claiming tile of this sub-phase is this one
            auto read_claims = [&](int k) {
                const unsigned long long key = base_key | (unsigned long long)k;
                const int nc = s_ncell;
                for (int i = tid; i <= nc; i += TB) {
                    const uint32_t id = i < nc ? clist[i] : 0u;
                    P.own[i < nc ? i + 1 : 0] = id == 0 || __ldcg(claims + id) == key;
                }
                __syncthreads();
            };
            // With one tile per CTA the box is staged while claiming.
            const bool single = per_color <= nblk;
            long long t_c0 = clock64();
            if (single) {
                if (blockIdx.x < per_color) {
                    setup_tile(blockIdx.x);
                    stage_box(blockIdx.x, true, 0u);
                }
            } else {
                // ---- claim the cells of every box this CTA will process
                for (int k = blockIdx.x; k < per_color; k += nblk) {
                    int tc[3];
                    tile_coords(k, tc);
                    int bdim[3], x0[3];
                    int box = 1;
                    for (int d = 0; d < D; ++d) {
                        const int L = g.dims[d];
                        const int b0 = tile_begin(tc[d], L, tg.nt[d]), b1 = tile_begin(tc[d] + 1, L, tg.nt[d]);
                        x0[d] = b0 + tg.off[d];
                        bdim[d] = b1 - b0 + 2;
                        box *= bdim[d];
                    }
                    const unsigned long long key = base_key | (unsigned long long)k;
                    const uint32_t stamp = stamp_of(k);
                    for (int q = tid; q < box; q += TB) {
                        int r = q, gf = 0;
                        for (int d = D - 1; d >= 0; --d) {
                            const int i = r % bdim[d];
                            r /= bdim[d];
                            int x = x0[d] + i - 1;
                            if (g.periodic) { x %= g.dims[d]; if (x < 0) x += g.dims[d]; }
                            gf += (x + 1) * (int)g.strides[d];
                        }
                        const uint32_t id = __ldcg(g.sigma + gf);
                        if (id && reg_first(id, stamp)) atomicMin(claims + id, key);
                    }
                    __syncthreads();
                }
            }
            const long long t_c1 = clock64();
            if (!grid_sync(bar, arrivals, bar_epoch)) { alive = false; break; }
            const long long t_c2 = clock64();
            ct.tick(TC_SYNC, t_c2 - t_c0);
            ct.tick(TC_CLAIM, t_c1 - t_c0);
            ct.tick(TC_BAR1, t_c2 - t_c1);
            // ---- process the tiles
            for (int k = blockIdx.x; k < per_color; k += nblk) {
                long long t_s0 = clock64();
                if (!single) {
                    setup_tile(k);
                    stage_box(k, false, 512u);  // a stamp distinct from the claim pass over this box
                    __syncthreads();
                }
                if (tid == 0) s_nchg = 0;
                read_claims(k);
                const unsigned long long key = base_key | (unsigned long long)k;
                (void)key;
                int box = 1;
                for (int d = 0; d < D; ++d) box *= s_box_dims[d];
                long long t_p0 = clock64();
                ct.tick(TC_STAGE, t_p0 - t_s0);
                // Site-colour passes of this tile, in the order staged with the
                // box. Every pass is first built at once from the state the
                // tile starts with (candidates, their neighbour halves and
                // first decisions): sigma and the cells change only through
                // commits, so while no pass has committed those builds are
                // exactly what building each pass in turn would give. A pass
                // without an accepting candidate needs no resolution (every
                // candidate is a final reject); the first pass that commits
                // ends the speculation, and each later pass is built again
                // after the one before it.
                //
                // The local sites of pass pi have colour sc_d on every axis d:
                // the parity, or (odd periodic axis) 2 for the last coordinate
                // L-1, whose neighbour across the wrap (0) has its parity. Per
                // axis they are first_a + 2i for i < cnt_a, then (past the
                // wrap) base_b + 2(i - cnt_a).
                if (tid < n_cls) {
                    int sc = sperm[tid];
                    int n_class = 1;
                    int* pg = s_pg[tid];
                    for (int d = 0; d < D; ++d) {
                        const int Ld = g.dims[d];
                        const int nc_d = ODD ? s_ncls[d] : 2;
                        const int want = ODD ? sc % nc_d : (sc >> d) & 1;
                        if (ODD) sc /= nc_d;
                        const int g0 = s_g0[d];
                        const int tc = s_tcnt[d];
                        int cnt, base, cnt_a, base_b;
                        if (nc_d == 2) {
                            const int first = (want - (g0 & 1)) & 1;  // first local offset with that parity
                            base = first;
                            cnt = tc > first ? (tc - first + 1) / 2 : 0;
                            cnt_a = cnt;
                            base_b = 0;
                        } else {
                            const int w = Ld - g0;  // local offsets before the wrap: g0 + i <= L - 1
                            if (want == 2) {
                                base = w - 1;
                                cnt = cnt_a = w - 1 < tc ? 1 : 0;
                                base_b = 0;
                            } else {
                                const int end_a = w - 1 < tc ? w - 1 : tc;  // g0 + i < L - 1
                                const int first = (want - (g0 & 1)) & 1;
                                base = first;
                                cnt_a = end_a > first ? (end_a - first + 1) / 2 : 0;
                                base_b = w + want;  // past the wrap: g = i - w
                                cnt = cnt_a + (tc > base_b ? (tc - base_b + 1) / 2 : 0);
                            }
                        }
                        pg[4 * d + 0] = cnt;
                        pg[4 * d + 1] = base;
                        pg[4 * d + 2] = cnt_a;
                        pg[4 * d + 3] = base_b;
                        n_class *= cnt;
                    }
                    s_pn[tid] = n_class;
                    s_pcnt[tid] = 0;
                    s_pacc[tid] = 0;
                    s_pguard[tid] = 0;
                    s_pnonnull[tid] = 0;
                    s_ptopo[tid] = 0;
                    s_pdef[tid] = 0;
                }
                __syncthreads();
                if (tid == 0) {
                    int acc = 0;
                    for (int q = 0; q < n_cls; ++q) { s_pfx[q] = acc; acc += s_pn[q]; }
                    s_pfx[n_cls] = acc;
                }
                __syncthreads();
                // One site j of pass pi: a candidate goes to slot atomicAdd(cnt)
                // of the slice at candidate `off` (capacity `cap`; beyond it the
                // pass overflows and is built again with the whole storage).
                // `spec`: event counts go to the pass's shared counters (used
                // only if the build is used), else to this thread's counters.
                auto build_site = [&](int pi, int j, int off, int cap, int* cnt, bool spec) {
                    const int* pg = s_pg[pi];
                    int r = j, t = 0;
                    int xg[3] = {0, 0, 0};
                    for (int d = D - 1; d >= 0; --d) {
                        const int c_d = pg[4 * d];
                        const int i = r % c_d;
                        r /= c_d;
                        const int li = !ODD || i < pg[4 * d + 2] ? pg[4 * d + 1] + 2 * i
                                                                : pg[4 * d + 3] + 2 * (i - pg[4 * d + 2]);
                        t += (li + 1) * (int)lsd.strides[d];
                        int x = s_g0[d] + li;  // global interior coordinate
                        if (x >= g.dims[d]) x -= g.dims[d];
                        xg[d] = x;
                    }
                    // this MCS's draw of the site (site_draw keyed by the global
                    // flat index); testing every copy neighbour first to skip
                    // the draw of null attempts measured 3 % slower on the
                    // 512^2 sorting lattice
                    const uint32_t L = P.sig[t];
                    int gf = 0;
                    for (int d = 0; d < D; ++d) gf += (xg[d] + 1) * (int)g.strides[d];
                    const uint4 rd = site_draw(g.seed, mcs, (uint32_t)gf);
                    const int kd = (int)(((unsigned long long)rd.x * (unsigned)g.n_copy) >> 32);
                    const uint32_t G = P.sig[t + s_coff[kd]];
                    if (L == G) return;
                    if (spec) atomicAdd(&s_pnonnull[pi], 1); else ct.nonnull++;
                    if (!P.own[L] || !P.own[G]) {
                        if (spec) atomicAdd(&s_pdef[pi], 1); else ct.deferred++;
                        return;
                    }
                    if (!tile_simple<D>(P.sig, s_toff, t, L, g.table2d, t3)) {
                        if (spec) atomicAdd(&s_ptopo[pi], 1); else ct.topo++;
                        return;
                    }
                    const int pos = atomicAdd(cnt, 1);
                    if (pos >= cap) return;
                    const int c = off + pos;
                    P.b_site[c] = (uint32_t)t;
                    P.b_cells[c] = L | (G << 16);
                    P.b_key[c] = (mix32((uint32_t)j * 0x9E3779B9u ^ s_pkey[pi]) & 0xFFFFC000u) | (uint32_t)j;
                    P.b_gf[c] = (uint32_t)gf;
                    P.b_z[c] = rd.z;
                    P.b_xy[c] = (uint32_t)xg[0] | ((uint32_t)xg[1] << 16);
                    if (D > 2) P.b_x2[c] = (uint16_t)xg[2];
                    uint32_t fl = (uint32_t)kd | T_PEND;
                    // the neighbour half of the decision, fixed for the pass
                    const NeighbourPart nb = decide_neighbours<NE, uint16_t, int>(lsd, P.sig, P.adh, s_eoff, t, L, G);
                    P.b_adh[c] = nb.adh;
                    P.b_sabs[c] = nb.sabs;
                    P.b_dl[c] = (int16_t)((nb.dl & 0xFF) | ((nb.dg & 0xFF) << 8));
                    // the first decision, on the volumes and interfaces before
                    // any commit of the pass (TileProc::evaluate, made here)
                    if (L != 0 && P.vol[L] <= lsd.min_cell_volume) {
                        fl |= T_GUARD;
                        atomicAdd(&s_pguard[pi], 1);
                    } else {
                        const TileDraw draw{g.seed, mcs, (uint32_t)gf, rd.z};
                        int rr;
                        if constexpr (MODES) {
                            rr = P.decide_modes_staged(t, t + s_coff[kd], L, G, mcs, draw, nb) ? 1 : 0;
                        } else {
                            rr = decide_cells(lsd, nb, P.adh[L], P.adh[G], P.vol, P.itf, L, G, draw);
                            if (rr < 0) rr = decide_exact<NE, uint16_t>(lsd, P.sig, P.adh, P.vol, P.itf, t, L, G, draw) ? 1 : 0;
                        }
                        if (rr) {
                            fl |= T_ACC;
                            s_pacc[pi] = 1;
                        }
                    }
                    P.b_flags[c] = fl;
                };
                const int ncap = TCMAX / n_cls;  // candidates per pass while speculating
                {
                    const long long tb0 = clock64();
                    const int total = s_pfx[n_cls];
                    for (int j0 = 0; j0 < total; j0 += TB) {
                        const int j = j0 + tid;
                        if (j >= total) break;
                        int pi = 0;
                        while (pi + 1 < n_cls && s_pfx[pi + 1] <= j) ++pi;
                        build_site(pi, j - s_pfx[pi], pi * ncap, ncap, &s_pcnt[pi], true);
                    }
                    __syncthreads();
                    ct.tick(TC_BUILD, clock64() - tb0);
                }
                bool spec = true;
                for (int pi = 0; pi < n_cls; ++pi) {
                    const int n_class = s_pn[pi];
                    int n, off;
                    bool acc;
                    uint32_t guards;
                    if (spec && s_pcnt[pi] <= ncap) {
                        // the speculative build of this pass stands
                        n = s_pcnt[pi];
                        off = pi * ncap;
                        acc = s_pacc[pi] != 0;
                        guards = (uint32_t)s_pguard[pi];
                        if (tid == 0) {
                            ct.nonnull += (uint32_t)s_pnonnull[pi];
                            ct.topo += (uint32_t)s_ptopo[pi];
                            ct.deferred += (uint32_t)s_pdef[pi];
                        }
                    } else {
                        // built again on the state the earlier passes left
                        spec = false;
                        const long long tb0 = clock64();
                        if (tid == 0) { s_n = 0; s_pacc[pi] = 0; s_pguard[pi] = 0; }
                        __syncthreads();
                        for (int j = tid; j < n_class; j += TB) build_site(pi, j, 0, TCMAX, &s_n, false);
                        __syncthreads();
                        n = min(s_n, TCMAX);
                        off = 0;
                        acc = s_pacc[pi] != 0;
                        guards = (uint32_t)s_pguard[pi];
                        ct.tick(TC_BUILD, clock64() - tb0);
                    }
                    P.at(off);
                    if (!acc) {
                        // no candidate accepts: all are final rejects
                        if (tid == 0) {
                            ct.guard += guards;
                            ct.evaluated += (uint32_t)n - guards;
                        }
                    } else {
                        spec = false;  // this pass commits
                        if (n > 64) {
                            P.resolve(n, mcs, ct);
                            ct.wide++;
                        } else {
                            if (tid < 32) {
                                if (n > 32) P.template resolve_warp<2>(n, mcs, ct);
                                else P.template resolve_warp<1>(n, mcs, ct);
                            }
                        }
                    }
                    // every thread has read this pass's counters before the
                    // next (re)build resets shared state
                    __syncthreads();
                    attempts += tid == 0 ? (unsigned long long)n_class : 0ull;
                    tile_passes += tid == 0 ? 1ull : 0ull;
                }
                long long t_w0 = clock64();
                ct.tick(TC_PASS, t_w0 - t_p0);
                // write back the sites commits changed (and their periodic
                // mirrors), or every tile site if the list overflowed, and
                // the owned cells
                const int nchg = s_nchg;
                if (nchg <= TCHG) {
                    for (int k2 = tid; k2 < nchg; k2 += TB) {
                        const int q = (int)P.chg[k2];
                        int xg[3];
                        P.gflat_of_box(q, xg);
                        const uint32_t sl = P.sig[q];
                        write_site<D, uint32_t>(g, g.sigma, xg, sl ? clist[sl - 1] : 0u);
                    }
                } else for (int q = tid; q < box; q += TB) {
                    int r = q;
                    int li[3];
                    bool interior = true;
                    for (int d = D - 1; d >= 0; --d) {
                        li[d] = r % s_box_dims[d];
                        r /= s_box_dims[d];
                        if (li[d] == 0 || li[d] == s_box_dims[d] - 1) interior = false;
                    }
                    if (interior) {
                        const uint32_t sl = P.sig[q];
                        int xg[3];
                        P.gflat_of_box(q, xg);
                        write_site<D, uint32_t>(g, g.sigma, xg, sl ? clist[sl - 1] : 0u);
                    }
                }
                __syncthreads();
                for (int i = tid; i < s_ncell; i += TB) {
                    const uint32_t id = clist[i];
                    const int sl = i + 1;
                    if (P.own[sl] && P.mod[sl]) {
                        __stcg(g.volume + id, P.vol[sl]);
                        __stcg(g.interface + id, P.itf[sl]);
                        if (i < cl_cap) {
                            for (int d = 0; d < D; ++d) __stcg((long long*)g.sum_pos + (int64_t)id * D + d, P.ssp[i * D + d]);
                            for (int d = 0; d < D * D; ++d)
                                __stcg((long long*)g.sum_outer + (int64_t)id * D * D + d, P.sso[i * D * D + d]);
                        }
                    }
                }
                __syncthreads();
                ct.tick(TC_STAGE, clock64() - t_w0);
            }
            long long t_b0 = clock64();
            if (!grid_sync(bar, arrivals, bar_epoch)) { alive = false; break; }
            ct.tick(TC_SYNC, clock64() - t_b0);
            ct.tick(TC_BAR2, clock64() - t_b0);
        }
    }
    // statistics: every site was attempted once per completed MCS
    atomicAdd(&sstat[1], ct.nonnull);
    atomicAdd(&sstat[2], ct.topo);
    atomicAdd(&sstat[3], ct.guard);
    atomicAdd(&sstat[4], ct.evaluated);
    atomicAdd(&sstat[5], ct.accepted);
    atomicAdd(&sstat[6], ct.deferred);
    atomicAdd(&sstat[0], attempts);
    __syncthreads();
    if (tid < 6) atomicAdd(&g.stats[tid], sstat[tid]);
    if (tid == 0) {
        atomicAdd(&g.stats[CPM_STAT_ROUNDS], ct.rounds);
        atomicAdd(&g.stats[CPM_STAT_DEFERRED], sstat[6]);
        atomicAdd(&g.stats[CPM_STAT_CYC_PASSES], s_cyc[TC_PASS]);
        atomicAdd(&g.stats[CPM_STAT_CYC_STAGE], s_cyc[TC_STAGE]);
        atomicAdd(&g.stats[CPM_STAT_CYC_SYNC], s_cyc[TC_SYNC]);
        atomicAdd(&g.stats[CPM_STAT_CYC_BUILD], s_cyc[TC_BUILD]);
        atomicAdd(&g.stats[CPM_STAT_CYC_EVAL], s_cyc[TC_EVAL]);
        atomicAdd(&g.stats[CPM_STAT_CYC_FIX], s_cyc[TC_FIX]);
        atomicAdd(&g.stats[CPM_STAT_CYC_APPLY], s_cyc[TC_APPLY]);
        atomicAdd(&g.stats[CPM_STAT_WIDE_PASSES], ct.wide);
        atomicAdd(&g.stats[CPM_STAT_CYC_LOWER], s_cyc[TC_LOWER]);
        atomicAdd(&g.stats[CPM_STAT_CYC_CLAIM], s_cyc[TC_CLAIM]);
        atomicAdd(&g.stats[CPM_STAT_CYC_BAR_CLAIM], s_cyc[TC_BAR1]);
        atomicAdd(&g.stats[CPM_STAT_CYC_BAR_WRITE], s_cyc[TC_BAR2]);
        atomicAdd(&g.stats[CPM_STAT_PASSES], tile_passes);
        if (blockIdx.x == 0 && alive) simp->mcs = mcs0 + n_mcs;
        if (!alive) {
            atomicAdd(&g.stats[CPM_STAT_SPIN_TIMEOUTS], 1ull);
            if (g.error) atomicExch(g.error, 5);
        }
    }
}

// ---- host side -------------------------------------------------------
static int tiled_index(int D, int NE) {
    if (D == 2 && NE == 4) return 0;
    if (D == 2 && NE == 8) return 1;
    if (D == 3 && NE == 6) return 2;
    if (D == 3 && NE == 18) return 3;
    if (D == 3 && NE == 26) return 4;
    return -1;
}

// The kernel variants of the including unit: even site colouring in
// cpm_tiled.cu; odd periodic sides in cpm_tiled_odd.cu, which includes this
// file with CPM_TILED_ODD_UNIT defined; the same two for the modes of the
// loop (Metropolis-Hastings, Act) in cpm_tiled_modes.cu and
// cpm_tiled_modes_odd.cu (CPM_TILED_MODES_UNIT). The four units build in
// parallel; the host entry points they share are compiled in cpm_tiled.cu
// only.
#if !defined(CPM_TILED_ODD_UNIT) && !defined(CPM_TILED_MODES_UNIT)
#define TILED_ODD false
#define TILED_MODES false
#define TILED_VARIANT(name) name##_even
#elif !defined(CPM_TILED_MODES_UNIT)
#define TILED_ODD true
#define TILED_MODES false
#define TILED_VARIANT(name) name##_odd
#elif !defined(CPM_TILED_ODD_UNIT)
#define TILED_ODD false
#define TILED_MODES true
#define TILED_VARIANT(name) name##_modes_even
#else
#define TILED_ODD true
#define TILED_MODES true
#define TILED_VARIANT(name) name##_modes_odd
#endif

// Shared-memory limit raised once per device (see prepare_resident_kernels).
cudaError_t TILED_VARIANT(prepare_tiled_kernels)() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    const int smem = 227 * 1024 - 4096;
    if ((e = cudaFuncSetAttribute(tiled_kernel<2, 4, TILED_ODD, TILED_MODES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
        (e = cudaFuncSetAttribute(tiled_kernel<2, 8, TILED_ODD, TILED_MODES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
        (e = cudaFuncSetAttribute(tiled_kernel<3, 6, TILED_ODD, TILED_MODES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
        (e = cudaFuncSetAttribute(tiled_kernel<3, 18, TILED_ODD, TILED_MODES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
        (e = cudaFuncSetAttribute(tiled_kernel<3, 26, TILED_ODD, TILED_MODES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
        return e;
    if (dev >= 0 && dev < 64) done[dev] = true;
    return cudaSuccess;
}

cudaError_t TILED_VARIANT(tiled_occupancy)(int D, int NE, size_t smem, int* per_sm) {
    *per_sm = 0;
    cudaError_t e = TILED_VARIANT(prepare_tiled_kernels)();
    if (e != cudaSuccess) return e;
#define TOCC(I, D_, NE_) \
    case I: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, tiled_kernel<D_, NE_, TILED_ODD, TILED_MODES>, TB, smem);
    switch (tiled_index(D, NE)) {
        TOCC(0, 2, 4)
        TOCC(1, 2, 8)
        TOCC(2, 3, 6)
        TOCC(3, 3, 18)
        TOCC(4, 3, 26)
        default: return cudaErrorInvalidValue;
    }
#undef TOCC
}

cudaError_t TILED_VARIANT(launch_tiled)(int D, int NE, SimDesc* d_sim, uint64_t n_mcs, const int* nt,
                                        void* d_barrier, unsigned long long* d_claims, uint32_t* d_registry,
                                        const uint64_t* d_t3, int max_box, int tables_in_smem, int barrier_extra,
                                        int cl_cap, int reg_smem, size_t smem, int grid, cudaStream_t st,
                                        int n_cells) {
    TileGrid tg;
    for (int d = 0; d < 3; ++d) { tg.nt[d] = d < D ? nt[d] : 1; tg.off[d] = 0; }
    tg.colors = 1 << D;
    BarrierState* bar = (BarrierState*)d_barrier;
    // in HBM unless reg_smem: grid x (n_cells + 1) stamps, then as many slots
    uint32_t* seen_all = d_registry;
    uint32_t* slot_all = d_registry ? d_registry + (size_t)grid * (size_t)(n_cells + 1) : nullptr;
#define TLAUNCH(I, D_, NE_)                                                                                 \
    case I: {                                                                                               \
        auto k = tiled_kernel<D_, NE_, TILED_ODD, TILED_MODES>;                                                           \
        cudaError_t e = TILED_VARIANT(prepare_tiled_kernels)();                                             \
        if (e != cudaSuccess) return e;                                                                     \
        void* args[] = {(void*)&d_sim, (void*)&n_mcs, (void*)&tg, (void*)&bar, (void*)&d_claims, (void*)&d_t3, \
                        (void*)&max_box, (void*)&tables_in_smem, (void*)&barrier_extra, (void*)&cl_cap,    \
                        (void*)&reg_smem, (void*)&seen_all, (void*)&slot_all};                              \
        return cudaLaunchCooperativeKernel((const void*)k, dim3(grid), dim3(TB), args, smem, st);            \
    }
    switch (tiled_index(D, NE)) {
        TLAUNCH(0, 2, 4)
        TLAUNCH(1, 2, 8)
        TLAUNCH(2, 3, 6)
        TLAUNCH(3, 3, 18)
        TLAUNCH(4, 3, 26)
        default: return cudaErrorInvalidValue;
    }
#undef TLAUNCH
}

#ifdef CPM_TILED_MAIN_UNIT
bool tiled_plan(int D, const int* dims, int periodic, int* nt, int* max_box) {
    (void)periodic;  // odd periodic axes take a third site colour in the kernel
    int box = 1, klass = 1;
    // Tiles per axis: as many as keep one tile per CTA on 152 SMs (n^D / 2^D
    // tiles per colour: n <= 24 in 2D, n <= 10 in 3D), while tiles stay at
    // least 14 (2D) or 8 (3D) sites wide; narrower tiles let cells span two
    // tiles of one colour, whose moves are then deferred. (Measured on 3D
    // organoids: 64^3 goes from 0.33 to 0.63 G attempts/s with 8 tiles per
    // axis instead of 4; 96^3 and 128^3 peak at 8-10.)
    const int wmin = D == 2 ? 14 : 8, nmax = D == 2 ? 24 : 10;
    for (int d = 0; d < D; ++d) {
        const int L = dims[d];
        int n = L / wmin < nmax ? L / wmin : nmax;
        if (n & 1) n -= 1;
        if (n < 2) return false;
        nt[d] = n;
        const int tmax = (L + n - 1) / n;
        box *= tmax + 2;
        klass *= (tmax + 1) / 2;
    }
    *max_box = box;
    // box slots are 16-bit: at most 65535 cells in a box
    return box <= TMAX_BOX && box <= 65535 && klass <= TCMAX;
}

size_t tiled_smem_bytes(int max_box, int n_cells, int cl_cap, int D, int reg_smem) {
    return tile_shared(max_box, n_cells, cl_cap, D, reg_smem != 0).total;
}
int tiled_block() { return TB; }

cudaError_t prepare_tiled_kernels() {
    cudaError_t e = prepare_tiled_kernels_even();
    if (e == cudaSuccess) e = prepare_tiled_kernels_odd();
    if (e == cudaSuccess) e = prepare_tiled_kernels_modes_even();
    if (e == cudaSuccess) e = prepare_tiled_kernels_modes_odd();
    return e;
}

cudaError_t tiled_occupancy(int D, int NE, int odd, int modes, size_t smem, int* per_sm) {
    if (modes) return odd ? tiled_occupancy_modes_odd(D, NE, smem, per_sm) : tiled_occupancy_modes_even(D, NE, smem, per_sm);
    return odd ? tiled_occupancy_odd(D, NE, smem, per_sm) : tiled_occupancy_even(D, NE, smem, per_sm);
}

cudaError_t launch_tiled(int D, int NE, int odd, int modes, SimDesc* d_sim, uint64_t n_mcs, const int* nt,
                         void* d_barrier, unsigned long long* d_claims, uint32_t* d_registry, const uint64_t* d_t3,
                         int max_box, int tables_in_smem, int barrier_extra, int cl_cap, int reg_smem, size_t smem,
                         int grid, cudaStream_t st, int n_cells) {
    auto* fn = modes ? (odd ? launch_tiled_modes_odd : launch_tiled_modes_even)
                     : (odd ? launch_tiled_odd : launch_tiled_even);
    return fn(D, NE, d_sim, n_mcs, nt, d_barrier, d_claims, d_registry, d_t3, max_box, tables_in_smem, barrier_extra,
              cl_cap, reg_smem, smem, grid, st, n_cells);
}
#endif

#undef TILED_ODD
#undef TILED_MODES
#undef TILED_VARIANT

}  // namespace cpmgpu
