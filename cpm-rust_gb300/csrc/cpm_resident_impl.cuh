// Shared-memory-resident sweep: one CTA owns one whole simulation.
//
// The halo-padded sigma lattice (16-bit ids), the per-cell volume and
// interface and the candidate lists of a colour pass all live in shared
// memory for the whole run plan; only the unwrapped position sums (touched
// by accepted moves alone) and the run-window outputs go to global memory.
//
// A colour pass (sites pairwise >= 2 apart, so no attempt reads a site
// another attempt of the pass writes) is resolved exactly as if its
// candidates were applied one by one in a fixed priority order
// (deterministic hash of the site's class index), each seeing the exact
// current volume and interface of its two cells:
//   1. build  — early-out and simple-point test (functions of sigma only);
//   2. speculate — every candidate evaluates the FP64 Delta-H and the
//      Metropolis test on the current V/I;
//   3. finalise — a shared-memory fixpoint marks candidate m final when
//      every lower-priority candidate on either of its cells is final and
//      rejected (so m's evaluation used exactly the state it would see);
//      final accepts are then pairwise cell-disjoint and commit in
//      parallel; candidates on cells that changed are re-evaluated and the
//      fixpoint repeats.
// Rejections are the common outcome (most copies cost energy), so one
// round usually finalises long chains of them; the number of rounds is the
// depth of chained accepts, not the number of candidates per cell.
//
// Reference semantics per attempt: monte_carlo.rs:52-145; run window:
// output.rs:434-468.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <type_traits>

#include "cpm_common.h"
#include "cpm_device.cuh"
#include "cpm_kernels.h"

namespace cpmgpu {

// Two block sizes: 512 threads (one CTA per SM) for simulations whose
// shared state needs more than half an SM, 256 threads with half the
// candidate capacity for smaller ones, so that two share an SM and hide
// each other's barrier latency. Which one a simulation uses depends only on
// its own size (resident_variant).
template <int BS>
struct ResCfg {
    static constexpr int CMAX = BS == 512 ? 2048 : 1024;   // candidate slots of one chunk
    static constexpr int CHUNK = BS == 512 ? 8192 : 4096;  // sites per chunk (halved while a chunk overflows CMAX)
};

// Active blocks: the lattice is cut into blocks of ABS^D sites (8 x 8 in
// 2D, 4 x 4 x 4 in 3D); a block is active when one of its sites may hold a
// non-null attempt (a copy neighbour with another cell). A bitmap of at
// most ACT_MAX blocks lives in shared memory; lattices with more blocks
// always take the plain build.
constexpr int ACT_WORDS = 64;
constexpr int ACT_MAX = ACT_WORDS * 32;
template <int D>
struct ActGeom {
    static constexpr int B = D == 2 ? 8 : 4;          // block side
    static constexpr int S = D == 2 ? 16 : 8;         // sites of one colour class in a block ((B/2)^D)
    static constexpr int SH = D == 2 ? 2 : 1;         // log2(B/2): sub-index bits per axis
};

// flag bits of a candidate
enum : uint32_t {
    F_K = 7u,           // copy direction (bits 0..2)
    F_ACC = 1u << 3,    // current evaluation accepts
    F_PEND = 1u << 4,   // not yet finalised
    F_FIN = 1u << 5,    // final in this round's fixpoint
    F_GUARD = 1u << 6,  // volume guard rejects
    F_DONE = 1u << 7,   // committed this round (clears dirty marks)
};

struct ResLayout {
    uint32_t sig, vol, itf, b0, b1, adh, dirty, c_site, c_key, c_cells, c_flags, c_dl, total;
};

__host__ __device__ inline uint32_t res_take(uint32_t& off, uint64_t bytes) {
    const uint32_t o = off;
    off = (uint32_t)((off + bytes + 15) & ~(uint64_t)15);
    return o;
}

__host__ __device__ inline ResLayout res_layout(int64_t n_padded, int n_cells, int CMAX) {
    ResLayout L;
    uint32_t off = 0;
    const uint64_t n1 = (uint64_t)n_cells + 1;
    L.sig = res_take(off, (uint64_t)n_padded * 2);
    L.vol = res_take(off, n1 * 4);
    L.itf = res_take(off, n1 * 4);
    L.b0 = res_take(off, n1 * 4);
    L.b1 = res_take(off, n1 * 4);
    L.adh = res_take(off, n1 * 2);
    L.dirty = res_take(off, n1);
    L.c_site = res_take(off, CMAX * 4);
    L.c_key = res_take(off, CMAX * 4);
    L.c_cells = res_take(off, CMAX * 4);
    L.c_flags = res_take(off, CMAX * 4);
    L.c_dl = res_take(off, CMAX * 2);
    L.total = off;
    return L;
}

struct PassInfoR {
    int cnt[3], base[3], step[3], n;
    // a reciprocal of cnt: idx / cnt == (idx * mg) >> 32 whenever
    // idx * cnt < 2^32 (every class index of a resident lattice)
    unsigned long long mg[3];
};

__device__ __forceinline__ void make_pass_r(const SimDesc& s, int color, PassInfoR& p) {
    int c = color;
    p.n = 1;
    for (int d = s.D - 1; d >= 0; --d) {
        const int cd = c % s.ncol[d];
        c /= s.ncol[d];
        if (cd == 2) { p.base[d] = s.dims[d] - 1; p.step[d] = 0; p.cnt[d] = 1; }
        else { p.base[d] = cd; p.step[d] = 2; p.cnt[d] = s.lim[d] > cd ? (s.lim[d] - cd + 1) / 2 : 0; }
        p.n *= p.cnt[d];
    }
    for (int d = s.D; d < 3; ++d) { p.cnt[d] = 1; p.base[d] = 0; p.step[d] = 0; }
    // (2^32 - 1) / cnt + 1 equals floor(2^32 / cnt) + 1 unless cnt is a power
    // of two, where it is 2^32 / cnt exactly: both give exact quotients
    for (int d = 0; d < 3; ++d) p.mg[d] = p.cnt[d] > 0 ? (unsigned long long)(0xFFFFFFFFu / (unsigned)p.cnt[d]) + 1ull : 0ull;
}

template <int D>
__device__ __forceinline__ int site_r(const SimDesc& s, const PassInfoR& p, int idx, int* x) {
    int f = 0;
#pragma unroll
    for (int d = D - 1; d >= 0; --d) {
        const int q = (int)(((unsigned long long)(unsigned)idx * p.mg[d]) >> 32);
        const int i = idx - q * p.cnt[d];
        idx = q;
        x[d] = p.base[d] + p.step[d] * i;
        f += (x[d] + 1) * (int)s.strides[d];
    }
    return f;
}

struct CountersR {
    unsigned long long attempts, nonnull, topo, guard, evaluated, accepted, rounds, iters, c_build, c_resolve;
};

template <int BLOCK>
__device__ double block_sum_r(double v, double* scratch) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < BLOCK / 32; ++w) t += scratch[w];
        scratch[0] = t;
    }
    __syncthreads();
    const double t = scratch[0];
    __syncthreads();
    return t;
}

// Global energy of the resident state (each unordered pair of different
// neighbouring cells contributes J once; volume and interface terms).
template <int D, int NE, int RB>
__device__ double res_energy(const SimDesc& s, const uint16_t* sig, const uint32_t* vol, const uint32_t* itf,
                             const uint16_t* adh, double* scratch) {
    const int nt1 = s.n_types + 1;
    double ea = 0.0;
    for (int q = threadIdx.x; q < (int)s.n_sites; q += RB) {
        int x[3];
        int r = q, f = 0;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
            x[d] = r % s.dims[d];
            r /= s.dims[d];
            f += (x[d] + 1) * (int)s.strides[d];
        }
        const uint32_t c = sig[f];
        const int ci = adh[c];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            bool count = (s.energy_pos_mask >> k) & 1u;
            if (!count && !s.periodic) {
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const int y = x[d] + s.energy_vec[k][d];
                    if (y < 0 || y >= s.dims[d]) count = true;
                }
            }
            if (!count) continue;
            const uint32_t n = sig[f + (int)s.energy_off[k]];
            if (n != c) ea += s.J[ci * nt1 + adh[n]];
        }
    }
    double ev = 0.0, ei = 0.0;
    for (int id = 1 + threadIdx.x; id <= s.n_cells; id += RB) {
        const int ty = adh[id] - 1;
        ev += quad_term(s.lambda_v[ty], s.target_v[ty], (double)vol[id]);
        ei += quad_term(s.lambda_i[ty], s.target_i[ty], (double)itf[id]);
    }
    ev = block_sum_r<RB>(ev, scratch);
    ei = block_sum_r<RB>(ei, scratch);
    ea = block_sum_r<RB>(ea, scratch);
    return (ev + ei) + ea;
}

// MODES: the simulations use Metropolis-Hastings acceptance or the Act term
// (decide_modes; compiled as separate kernels, so that the Metropolis
// kernels keep their registers).
template <int D, int NE, int RB, bool MODES>
struct Resident {
    static constexpr int CMAX = ResCfg<RB>::CMAX;
    static constexpr int CHUNK = ResCfg<RB>::CHUNK;
    const SimDesc& s;
    uint16_t* sig;
    uint32_t *vol, *itf, *b0, *b1;
    uint16_t* adh;
    uint8_t* dirty;
    uint32_t *c_site, *c_key, *c_cells, *c_flags;
    int16_t* c_dl;  // dl in the low byte, dg in the high byte
    const uint64_t* t3;
    int* s_n;
    int* s_flag;
    uint32_t* act;  // active-block bitmap (ACT_WORDS words)
    int* apfx;      // active blocks before each bitmap word (ACT_WORDS + 1)
    int nb[3];      // blocks per axis (0: the lattice has more than ACT_MAX blocks)

    __device__ __forceinline__ int block_of(const int* x) const {
        constexpr int B = ActGeom<D>::B;
        int b = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) b = b * nb[d] + x[d] / B;
        return b;
    }
    __device__ __forceinline__ void mark(const int* x) { const int b = block_of(x); atomicOr(&act[b >> 5], 1u << (b & 31)); }
    // After sigma[x] changed: x and its copy neighbours may now have a
    // non-null attempt (periodic neighbours wrap; fixed ones outside are the
    // medium halo, which never changes).
    __device__ void mark_around(const int* x) {
        if (nb[0] == 0) return;
        mark(x);
        for (int d = 0; d < D; ++d)
            for (int sg = -1; sg <= 1; sg += 2) {
                int y[3] = {x[0], D > 1 ? x[1] : 0, D > 2 ? x[2] : 0};
                y[d] += sg;
                if (y[d] < 0 || y[d] >= s.dims[d]) {
                    if (!s.periodic) continue;
                    y[d] = y[d] < 0 ? s.dims[d] - 1 : 0;
                }
                mark(y);
            }
    }
    // Rebuilds the bitmap from sigma (every thread; ends with a barrier).
    __device__ void rescan() {
        if (nb[0] == 0) return;
        for (int w = threadIdx.x; w < ACT_WORDS; w += RB) act[w] = 0u;
        __syncthreads();
        for (int q = threadIdx.x; q < (int)s.n_sites; q += RB) {
            int x[3] = {0, 0, 0}, r = q, f = 0;
#pragma unroll
            for (int d = D - 1; d >= 0; --d) {
                x[d] = r % s.dims[d];
                r /= s.dims[d];
                f += (x[d] + 1) * (int)s.strides[d];
            }
            if (!copy_uniform(s, sig, f, (uint32_t)sig[f])) mark(x);
        }
        __syncthreads();
    }

    // Evaluate candidate c on the current state (guard, Delta-H, Metropolis).
    __device__ void evaluate(int c, uint64_t mcs) {
        const int t = (int)c_site[c];
        const uint32_t cells = c_cells[c];
        const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
        uint32_t fl = c_flags[c] & ~(F_ACC | F_GUARD);
        if (L != 0 && vol[L] <= s.min_cell_volume) {
            fl |= F_GUARD;
        } else {
            int dl = 0, dg = 0;
            bool acc;
            if constexpr (MODES) {
                acc = decide_modes_sweep<NE>(s, sig, adh, vol, itf, t, t + s.copy_off[fl & F_K], L, G, mcs,
                                             PhiloxDraw{s.seed, mcs, (uint32_t)t}, dl, dg);
            } else {
                acc = decide_move<NE, uint16_t>(s, sig, adh, vol, itf, t, L, G, PhiloxDraw{s.seed, mcs, (uint32_t)t}, dl, dg);
            }
            if (acc) fl |= F_ACC;
            c_dl[c] = (int16_t)((dl & 0xFF) | ((dg & 0xFF) << 8));
        }
        c_flags[c] = fl;
    }

    __device__ void commit(int c, uint64_t mcs) {
        const int t = (int)c_site[c];
        const uint32_t cells = c_cells[c];
        const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
        const int16_t dd = c_dl[c];
        const int dl = (int)(int8_t)(dd & 0xFF), dg = (int)(int8_t)((dd >> 8) & 0xFF);
        int x[3];
        int f = t;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int q = f / (int)s.strides[d];
            f -= q * (int)s.strides[d];
            x[d] = q - 1;
        }
        commit_move<D, uint16_t>(s, sig, vol, itf, s.sum_pos, s.sum_outer, x, L, G, dl, dg);
        if constexpr (MODES) {
            if (s.act) s.birth[t] = (uint32_t)mcs;  // energy.rs:453-458
        }
        if (L) dirty[L] = 1;
        if (G) dirty[G] = 1;
        mark_around(x);
    }

    // The same outcome as resolve() for n <= 32 (K = 1) or n <= 64 (K = 2)
    // candidates, by one warp, candidate c = lane + 32 q: `lower` holds the
    // lower-priority candidates sharing a cell (the medium is not a cell);
    // a pending candidate is final once every lower pending one is a final
    // reject; final accepts are pairwise cell-disjoint and commit; a
    // pending candidate with a committed lower neighbour decides again.
    // Every candidate has been evaluated; b0 and b1 are free.
    template <int K>
    using Mask = typename std::conditional<K == 1, uint32_t, uint64_t>::type;
    template <int K>
    __device__ __forceinline__ static Mask<K> ballot_k(const bool (&p)[K]) {
        Mask<K> m = __ballot_sync(0xffffffffu, p[0]);
        if (K > 1) m |= (Mask<K>)__ballot_sync(0xffffffffu, p[K > 1 ? 1 : 0]) << (K > 1 ? 32 : 0);
        return m;
    }
    template <int K>
    __device__ void resolve_warp(int n, uint64_t mcs, CountersR& ct) {
        const int lane = threadIdx.x & 31;
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
            sh &= ~((Mask<K>)1 << (lane + 32 * q));
            Mask<K> lw = 0;
            while (sh) {
                const int j = K == 1 ? __ffs((uint32_t)sh) - 1 : __ffsll((long long)sh) - 1;
                sh &= sh - 1;
                if (c_key[j] < key[q]) lw |= (Mask<K>)1 << j;
            }
            lower[q] = lw;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < K; ++q) fl[q] = have[q] ? c_flags[lane + 32 * q] : 0u;
        Mask<K> pending = ballot_k<K>(have);
        while (pending) {
            bool mine[K], rej[K];
#pragma unroll
            for (int q = 0; q < K; ++q) {
                mine[q] = (pending >> (lane + 32 * q)) & 1u;
                rej[q] = (fl[q] & F_GUARD) || !(fl[q] & F_ACC);
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
                ct.iters += lane == 0;
                if (f2 == fin) break;
                fin = f2;
            }
            bool cm[K];
#pragma unroll
            for (int q = 0; q < K; ++q) {
                const bool is_fin = (fin >> (lane + 32 * q)) & 1u;
                cm[q] = is_fin && !rej[q];
                if (is_fin) {
                    if (fl[q] & F_GUARD) ct.guard++;
                    else ct.evaluated++;
                }
                if (cm[q]) {
                    commit(lane + 32 * q, mcs);
                    ct.accepted++;
                }
            }
            const Mask<K> committed = ballot_k<K>(cm);
            pending &= ~fin;
            ct.rounds += lane == 0;
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
        }
        // commit() marks the cells it changes dirty; clear those marks
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (Lc[q]) dirty[Lc[q]] = 0;
            if (Gc[q]) dirty[Gc[q]] = 0;
        }
        __syncwarp();
    }

    // Resolve the candidates [0, n) of one chunk in priority order.
    __device__ void resolve(int n, uint64_t mcs, CountersR& ct) {
        const int tid = threadIdx.x;
        bool any_acc = false;
        for (int c = tid; c < n; c += RB) {
            evaluate(c, mcs);
            any_acc |= (c_flags[c] & (F_ACC | F_GUARD)) == F_ACC;
        }
        if (!__syncthreads_or(any_acc)) {
            // no candidate accepts: every one is a final reject
            for (int c = tid; c < n; c += RB) {
                if (c_flags[c] & F_GUARD) ct.guard++;
                else ct.evaluated++;
            }
            ct.rounds += tid == 0;
            return;
        }
        if (n <= 64) {
            // one warp on register masks, no block barrier inside
            if (tid < 32) {
                if (n > 32) resolve_warp<2>(n, mcs, ct);
                else resolve_warp<1>(n, mcs, ct);
            }
            __syncthreads();
            return;
        }
        for (;;) {
            // ---- finality. A pending candidate is final unless an accepting
            // candidate lies in its lower closure (lower-key candidates
            // sharing a cell, transitively): then every candidate before it
            // in the sequential order leaves its cells as they are. Per cell,
            // T = the lowest key of an accepting or tainted candidate on it;
            // a candidate with a key above T on either cell is tainted and
            // lowers T on both; iterate until T is stable. Rejects add
            // nothing, so the iterations count cross-cell hops of accepts.
            for (int c = tid; c < n; c += RB) {
                if (!(c_flags[c] & F_PEND)) continue;
                const uint32_t cells = c_cells[c];
                if (cells & 0xFFFFu) b0[cells & 0xFFFFu] = 0xFFFFFFFFu;
                if (cells >> 16) b0[cells >> 16] = 0xFFFFFFFFu;
            }
            __syncthreads();
            for (int c = tid; c < n; c += RB) {
                const uint32_t fl = c_flags[c];
                if (!(fl & F_PEND) || !(fl & F_ACC) || (fl & F_GUARD)) continue;
                const uint32_t cells = c_cells[c], key = c_key[c];
                if (cells & 0xFFFFu) atomicMin(&b0[cells & 0xFFFFu], key);
                if (cells >> 16) atomicMin(&b0[cells >> 16], key);
            }
            for (;;) {
                __syncthreads();
                int changed = 0;
                for (int c = tid; c < n; c += RB) {
                    if (!(c_flags[c] & F_PEND)) continue;
                    const uint32_t cells = c_cells[c], key = c_key[c];
                    const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
                    const bool tainted = (L && key > b0[L]) || (G && key > b0[G]);
                    if (!tainted) continue;
                    if (L && atomicMin(&b0[L], key) > key) changed = 1;
                    if (G && atomicMin(&b0[G], key) > key) changed = 1;
                }
                ct.iters++;
                if (!__syncthreads_or(changed)) break;
            }
            // ---- apply the final candidates
            int left = 0;
            for (int c = tid; c < n; c += RB) {
                uint32_t fl = c_flags[c];
                if (!(fl & F_PEND)) continue;
                const uint32_t cells = c_cells[c], key = c_key[c];
                const uint32_t L = cells & 0xFFFFu, G = cells >> 16;
                if ((L && key > b0[L]) || (G && key > b0[G])) { left = 1; continue; }
                fl &= ~F_PEND;
                if (fl & F_GUARD) {
                    ct.guard++;
                } else {
                    ct.evaluated++;
                    if (fl & F_ACC) {
                        commit(c, mcs);
                        fl |= F_DONE;
                        ct.accepted++;
                    }
                }
                c_flags[c] = fl;
            }
            ct.rounds++;
            const int more = __syncthreads_or(left);
            if (!more) break;
            // ---- re-evaluate candidates whose cells changed, then clear the marks
            for (int c = tid; c < n; c += RB) {
                const uint32_t fl = c_flags[c];
                if (!(fl & F_PEND)) continue;
                const uint32_t cells = c_cells[c];
                if (dirty[cells & 0xFFFFu] || dirty[cells >> 16]) evaluate(c, mcs);
            }
            __syncthreads();
            for (int c = tid; c < n; c += RB) {
                uint32_t fl = c_flags[c];
                if (!(fl & F_DONE)) continue;
                const uint32_t cells = c_cells[c];
                dirty[cells & 0xFFFFu] = 0;
                dirty[cells >> 16] = 0;
                c_flags[c] = fl & ~F_DONE;
            }
            __syncthreads();
        }
        // clear the marks of the last round's commits
        for (int c = tid; c < n; c += RB) {
            const uint32_t fl = c_flags[c];
            if (!(fl & F_DONE)) continue;
            const uint32_t cells = c_cells[c];
            dirty[cells & 0xFFFFu] = 0;
            dirty[cells >> 16] = 0;
        }
        __syncthreads();
    }

    // Site j of a chunk (class index start + j) at padded index t: the
    // draw, the early-out, the connectivity test; a candidate keeps its
    // copy direction in k. (Testing all copy neighbours first to skip the
    // draw of null attempts costs more shared-memory loads than the draw
    // costs arithmetic: 13 % slower on dense 256^2 lattices. Sparse
    // lattices skip whole blocks instead.)
    __device__ __forceinline__ bool try_site(int t, uint64_t mcs, int& k, uint32_t& L, uint32_t& G,
                                             unsigned long long& nonnull, unsigned long long& topo) {
        L = sig[t];
        const uint4 r = site_draw(s.seed, mcs, (uint32_t)t);
        k = (int)(((unsigned long long)r.x * (unsigned)s.n_copy) >> 32);
        G = sig[t + (int)s.copy_off[k]];
        if (L == G) return false;
        ++nonnull;
        if (preserves_topology<D, uint16_t>(s, sig, t, L, s.table2d, t3)) return true;
        ++topo;
        return false;
    }
    __device__ __forceinline__ void add_candidate(bool cand, int j, int t, int k, uint32_t L, uint32_t G,
                                                  uint32_t pass_key) {
        const int lane = threadIdx.x & 31;
        const unsigned m = __ballot_sync(0xffffffffu, cand);
        int base = 0;
        if (lane == 0 && m) base = atomicAdd(s_n, __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (cand) {
            const int pos = base + __popc(m & ((1u << lane) - 1));
            if (pos < CMAX) {
                c_site[pos] = (uint32_t)t;
                c_cells[pos] = L | (G << 16);
                c_key[pos] = (mix32((uint32_t)j * 0x9E3779B9u ^ pass_key) & 0xFFFFC000u) | (uint32_t)j;
                c_flags[pos] = (uint32_t)k | F_PEND;
            }
        }
    }

    // One colour pass: chunks of the class in index order. A chunk whose
    // active blocks hold fewer than half its sites visits only their sites
    // of the class: every other site has copy neighbours of its own cell,
    // a null attempt that neither draws nor counts, so the candidates (and
    // their keys, from the class index) are those of the plain build.
    __device__ void pass(const PassInfoR& p, uint64_t mcs, uint32_t pass_key, CountersR& ct) {
        constexpr int B = ActGeom<D>::B, S = ActGeom<D>::S, SH = ActGeom<D>::SH;
        const int tid = threadIdx.x;
        const int lane = tid & 31;
        int start = 0;
        while (start < p.n) {
            int len = min(CHUNK, p.n - start);
            for (;;) {
                const long long t0 = clock64();
                int nact = 0;
                if (nb[0] > 0)
                    nact = __reduce_add_sync(0xffffffffu, (unsigned)(__popc(act[lane]) + __popc(act[lane + 32])));
                if (tid == 0) *s_n = 0;
                __syncthreads();
                unsigned long long nonnull = 0, topo = 0;
                if (nb[0] > 0 && 2 * nact * S < len) {
                    // the sites of the active blocks, spread over all
                    // threads: item q is site q % S of the (q / S)-th active
                    // block in bitmap order (word prefix sums in apfx)
                    if (tid < 32) {
                        const int c0 = __popc(act[lane]), c1 = __popc(act[lane + 32]);
                        int i0 = c0, i1 = c1;
                        for (int o = 1; o < 32; o <<= 1) {
                            const int y0 = __shfl_up_sync(0xffffffffu, i0, o), y1 = __shfl_up_sync(0xffffffffu, i1, o);
                            if (lane >= o) { i0 += y0; i1 += y1; }
                        }
                        const int tot0 = __shfl_sync(0xffffffffu, i0, 31);
                        apfx[lane] = i0 - c0;
                        apfx[lane + 32] = tot0 + i1 - c1;
                        if (lane == 31) apfx[64] = tot0 + i1;
                    }
                    __syncthreads();
                    const int total = apfx[64] * S;
                    for (int q0 = 0; q0 < total; q0 += RB) {
                        const int q = q0 + tid;
                        bool cand = false, valid = q < total;
                        int t = 0, k = 0, jj = 0;
                        uint32_t L = 0, G = 0;
                        if (valid) {
                            const int a = q / S, sub = q % S;
                            int lo = 0, hi = ACT_WORDS - 1;  // the word holding active block a
                            while (lo < hi) {
                                const int mid = (lo + hi + 1) >> 1;
                                if (apfx[mid] <= a) lo = mid; else hi = mid - 1;
                            }
                            int blk = lo * 32 + (int)__fns(act[lo], 0, a - apfx[lo] + 1);
                            int bc[3], jc = 0;
                            for (int d = D - 1; d >= 0; --d) { bc[d] = blk % nb[d]; blk /= nb[d]; }
                            for (int d = 0; d < D && valid; ++d) {
                                const int sd = (sub >> (SH * (D - 1 - d))) & ((1 << SH) - 1);
                                int i, x;
                                if (p.step[d] == 0) {
                                    i = 0;
                                    x = p.base[d];
                                    valid = sd == 0 && x >= B * bc[d] && x < B * bc[d] + B;
                                } else {
                                    const int lo2 = B * bc[d] > p.base[d] ? (B * bc[d] - p.base[d] + 1) >> 1 : 0;
                                    i = lo2 + sd;
                                    x = p.base[d] + 2 * i;
                                    valid = i < p.cnt[d] && x < B * bc[d] + B;
                                }
                                jc = jc * p.cnt[d] + i;
                                t += (x + 1) * (int)s.strides[d];
                            }
                            jj = jc - start;
                            valid = valid && jj >= 0 && jj < len;
                            if (valid) cand = try_site(t, mcs, k, L, G, nonnull, topo);
                        }
                        add_candidate(cand, jj, t, k, L, G, pass_key);
                    }
                } else {
                    for (int j0 = 0; j0 < len; j0 += RB) {
                        const int j = j0 + tid;
                        bool cand = false;
                        int t = 0, k = 0;
                        uint32_t L = 0, G = 0;
                        if (j < len) {
                            int x[3];
                            t = site_r<D>(s, p, start + j, x);
                            cand = try_site(t, mcs, k, L, G, nonnull, topo);
                        }
                        add_candidate(cand, j, t, k, L, G, pass_key);
                    }
                }
                __syncthreads();
                const int n = *s_n;
                __syncthreads();
                if (n > CMAX) { len >>= 1; continue; }  // retry this chunk with fewer sites
                ct.nonnull += nonnull;
                ct.topo += topo;
                const long long t1 = clock64();
                ct.c_build += t1 - t0;
                if (n > 0) resolve(n, mcs, ct);
                ct.c_resolve += clock64() - t1;
                break;
            }
            start += len;
        }
        (void)lane;
    }
};

template <int D, int NE, int RB, bool MODES>
__global__ void __launch_bounds__(RB, 512 / RB) resident_kernel(SimDesc* sims, const RunPlan* plans, int n_plans,
                                                                int* next_plan, const uint64_t* t3) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ SimDesc sd;
    __shared__ int s_plan, s_n, s_flag;
    __shared__ int perm[27], s_swap[27];
    __shared__ uint32_t s_act[ACT_WORDS];
    __shared__ int s_apfx[ACT_WORDS + 1];
    __shared__ PassInfoR pinfo;
    __shared__ double scratch[RB / 32];
    __shared__ unsigned long long sstat[10];
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_plan = atomicAdd(next_plan, 1);
        __syncthreads();
        const int pl = s_plan;
        __syncthreads();
        if (pl >= n_plans) return;
        const RunPlan plan = plans[pl];
        if (tid == 0) sd = sims[plan.sim];
        if (tid < 10) sstat[tid] = 0;
        __syncthreads();
        const ResLayout lay = res_layout(sd.n_padded, sd.n_cells, ResCfg<RB>::CMAX);
        Resident<D, NE, RB, MODES> R{sd,
                          (uint16_t*)(sm + lay.sig),
                          (uint32_t*)(sm + lay.vol),
                          (uint32_t*)(sm + lay.itf),
                          (uint32_t*)(sm + lay.b0),
                          (uint32_t*)(sm + lay.b1),
                          (uint16_t*)(sm + lay.adh),
                          (uint8_t*)(sm + lay.dirty),
                          (uint32_t*)(sm + lay.c_site),
                          (uint32_t*)(sm + lay.c_key),
                          (uint32_t*)(sm + lay.c_cells),
                          (uint32_t*)(sm + lay.c_flags),
                          (int16_t*)(sm + lay.c_dl),
                          t3,
                          &s_n,
                          &s_flag};
        R.act = s_act;
        R.apfx = s_apfx;
        {
            constexpr int B = ActGeom<D>::B;
            int nbt = 1;
            for (int d = 0; d < 3; ++d) {
                R.nb[d] = d < D ? (sd.dims[d] + B - 1) / B : 1;
                nbt *= R.nb[d];
            }
            // too many blocks, or the test switch: the plain build only
            if (nbt > ACT_MAX || (sd.sweep_flags & 1)) R.nb[0] = 0;
        }
        // ---- stage the state into shared memory
        for (int f = tid; f < (int)sd.n_padded; f += RB) R.sig[f] = (uint16_t)sd.sigma[f];
        for (int id = tid; id <= sd.n_cells; id += RB) {
            R.vol[id] = sd.volume[id];
            R.itf[id] = sd.interface[id];
            R.adh[id] = sd.adh_of[id];
            R.dirty[id] = 0;
        }
        __syncthreads();
        CountersR ct = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        uint64_t mcs = sd.mcs;
        R.rescan();
        auto one_mcs = [&](uint64_t m) {
            // commits only add active blocks; clear the stale ones now and then
            if ((m & 15u) == 0u && m != sd.mcs) R.rescan();
            // Fisher-Yates over the colours: the draws one per thread, then
            // the swaps
            if (tid > 0 && tid < sd.n_colors) {
                const uint4 r = aux_draw(sd.seed, m, TAG_ORDER, (uint32_t)tid, 0u);
                s_swap[tid] = (int)(((unsigned long long)r.x * (unsigned)(tid + 1)) >> 32);
            }
            __syncthreads();
            if (tid == 0) {
                const int nc = sd.n_colors;
                for (int c = 0; c < nc; ++c) perm[c] = c;
                for (int c = nc - 1; c > 0; --c) {
                    const int j = s_swap[c];
                    const int tmp = perm[c]; perm[c] = perm[j]; perm[j] = tmp;
                }
            }
            __syncthreads();
            for (int pi = 0; pi < sd.n_colors; ++pi) {
                if (tid == 0) make_pass_r(sd, perm[pi], pinfo);
                __syncthreads();
                const PassInfoR p = pinfo;
                const uint32_t pass_key = aux_draw(sd.seed, m, TAG_PASS, (uint32_t)pi, 0u).x;
                R.pass(p, m, pass_key, ct);
                __syncthreads();
            }
            ct.attempts += (tid == 0) ? (unsigned long long)sd.n_sites : 0ull;
        };
        // ---- run plan (output.rs:441-468)
        uint64_t burned = 0;
        int e_idx = 0;
        while (burned < plan.burn_in) {
            const uint64_t chunk = plan.interval < plan.burn_in - burned ? plan.interval : plan.burn_in - burned;
            for (uint64_t m = 0; m < chunk; ++m, ++mcs) one_mcs(mcs);
            burned += chunk;
            if (burned >= plan.energy_sample_start) {
                const double e = res_energy<D, NE, RB>(sd, R.sig, R.vol, R.itf, R.adh, scratch);
                if (tid == 0 && sd.energy_out) sd.energy_out[e_idx] = e;
                ++e_idx;
            }
        }
        for (int smp = 0; smp < plan.n_samples; ++smp) {
            for (uint64_t m = 0; m < plan.interval; ++m, ++mcs) one_mcs(mcs);
            const double e = res_energy<D, NE, RB>(sd, R.sig, R.vol, R.itf, R.adh, scratch);
            if (tid == 0 && sd.energy_out) sd.energy_out[e_idx + smp] = e;
            if (plan.write_samples) {
                const int n1 = sd.n_cells + 1;
                for (int id = tid; id < n1; id += RB) {
                    sd.sample_volume[(int64_t)smp * n1 + id] = R.vol[id];
                    sd.sample_interface[(int64_t)smp * n1 + id] = R.itf[id];
                    for (int d = 0; d < D; ++d)
                        sd.sample_sum_pos[((int64_t)smp * n1 + id) * D + d] = sd.sum_pos[(int64_t)id * D + d];
                    for (int d = 0; d < D * D; ++d)
                        sd.sample_sum_outer[((int64_t)smp * n1 + id) * D * D + d] = sd.sum_outer[(int64_t)id * D * D + d];
                }
            }
            if (plan.write_lattice && sd.sample_lattice) {
                for (int q = tid; q < (int)sd.n_sites; q += RB) {
                    int r = q, f = 0;
#pragma unroll
                    for (int d = D - 1; d >= 0; --d) {
                        f += (r % sd.dims[d] + 1) * (int)sd.strides[d];
                        r /= sd.dims[d];
                    }
                    sd.sample_lattice[(int64_t)smp * sd.n_sites + q] = R.sig[f];
                }
            }
            __syncthreads();
        }
        // ---- write the state back
        for (int f = tid; f < (int)sd.n_padded; f += RB) sd.sigma[f] = R.sig[f];
        for (int id = tid; id <= sd.n_cells; id += RB) {
            sd.volume[id] = R.vol[id];
            sd.interface[id] = R.itf[id];
        }
        atomicAdd(&sstat[CPM_STAT_ATTEMPTS], ct.attempts);
        atomicAdd(&sstat[CPM_STAT_NONNULL], ct.nonnull);
        atomicAdd(&sstat[CPM_STAT_TOPO_REJECT], ct.topo);
        atomicAdd(&sstat[CPM_STAT_GUARD_REJECT], ct.guard);
        atomicAdd(&sstat[CPM_STAT_EVALUATED], ct.evaluated);
        atomicAdd(&sstat[CPM_STAT_ACCEPTED], ct.accepted);
        atomicAdd(&sstat[9], ct.iters);
        __syncthreads();
        if (tid < 6) atomicAdd(&sd.stats[tid], sstat[tid]);
        if (tid == 0) {
            atomicAdd(&sd.stats[CPM_STAT_ROUNDS], ct.rounds);
            atomicAdd(&sd.stats[CPM_STAT_PASSES], (unsigned long long)(mcs - sd.mcs) * sd.n_colors);
            atomicAdd(&sd.stats[9], sstat[9]);
            atomicAdd(&sd.stats[CPM_STAT_CYC_RES_BUILD], ct.c_build);
            atomicAdd(&sd.stats[CPM_STAT_CYC_RES_RESOLVE], ct.c_resolve);
            sims[plan.sim].mcs = mcs;
        }
        __syncthreads();
        if (tid == 0 && sd.done_flag) {
            // every write of this plan (state, samples, counters) before the flag
            __threadfence_system();
            *(volatile uint32_t*)sd.done_flag = 1u;
        }
        __syncthreads();
    }
}

static int res_index(int D, int NE) {
    if (D == 2 && NE == 4) return 0;
    if (D == 2 && NE == 8) return 1;
    if (D == 3 && NE == 6) return 2;
    if (D == 3 && NE == 18) return 3;
    if (D == 3 && NE == 26) return 4;
    return -1;
}

// The kernel variants of the including unit: Metropolis in cpm_resident.cu;
// Metropolis-Hastings / Act in cpm_resident_modes.cu, which includes this
// file with CPM_RESIDENT_MODES_UNIT defined (two units build in parallel).
// The host entry points shared by both are compiled in cpm_resident.cu only.
#ifndef CPM_RESIDENT_MODES_UNIT
#define RES_MODES false
#define RES_VARIANT(name) name##_plain
#else
#define RES_MODES true
#define RES_VARIANT(name) name##_modes
#endif

// The kernels' shared-memory limit is raised once per device, before any
// launch: changing a function attribute while kernels run can wait for
// them, which would serialise launches on different streams.
cudaError_t RES_VARIANT(prepare_resident_kernels)() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    const int smem = (int)resident_smem_limit();
#define RES_ATTR(D_, NE_)                                                                                    \
    if ((e = cudaFuncSetAttribute(resident_kernel<D_, NE_, 256, RES_MODES>,                                  \
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)        \
        return e;                                                                                              \
    if ((e = cudaFuncSetAttribute(resident_kernel<D_, NE_, 512, RES_MODES>,                                  \
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)        \
        return e;
    RES_ATTR(2, 4)
    RES_ATTR(2, 8)
    RES_ATTR(3, 6)
    RES_ATTR(3, 18)
    RES_ATTR(3, 26)
#undef RES_ATTR
    if (dev >= 0 && dev < 64) done[dev] = true;
    return cudaSuccess;
}

cudaError_t RES_VARIANT(launch_resident)(int Dd, int NEd, int variant, SimDesc* d_sims, const RunPlan* d_plans,
                                         int n_plans, int* d_next, const uint64_t* d_t3, size_t smem, int grid,
                                         cudaStream_t st) {
    cudaError_t e = RES_VARIANT(prepare_resident_kernels)();
    if (e != cudaSuccess) return e;
#define RES_CASE(I, D_, NE_)                                                                                      \
    case I: {                                                                                                     \
        if (variant)                                                                                              \
            resident_kernel<D_, NE_, 256, RES_MODES><<<grid, 256, smem, st>>>(d_sims, d_plans, n_plans, d_next, d_t3); \
        else                                                                                                      \
            resident_kernel<D_, NE_, 512, RES_MODES><<<grid, 512, smem, st>>>(d_sims, d_plans, n_plans, d_next, d_t3); \
        break;                                                                                                    \
    }
    switch (res_index(Dd, NEd)) {
        RES_CASE(0, 2, 4)
        RES_CASE(1, 2, 8)
        RES_CASE(2, 3, 6)
        RES_CASE(3, 3, 18)
        RES_CASE(4, 3, 26)
        default: return cudaErrorInvalidValue;
    }
#undef RES_CASE
    return cudaGetLastError();
}

cudaError_t RES_VARIANT(resident_occupancy)(int Dd, int NEd, int variant, size_t smem, int* blocks_per_sm) {
    *blocks_per_sm = 1;
    cudaError_t e = RES_VARIANT(prepare_resident_kernels)();
    if (e != cudaSuccess) return e;
#define OCC_CASE(I, D_, NE_)                                                                                      \
    case I:                                                                                                       \
        return variant ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                          \
                             blocks_per_sm, resident_kernel<D_, NE_, 256, RES_MODES>, 256, smem)                  \
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                          \
                             blocks_per_sm, resident_kernel<D_, NE_, 512, RES_MODES>, 512, smem);
    switch (res_index(Dd, NEd)) {
        OCC_CASE(0, 2, 4)
        OCC_CASE(1, 2, 8)
        OCC_CASE(2, 3, 6)
        OCC_CASE(3, 3, 18)
        OCC_CASE(4, 3, 26)
        default: return cudaErrorInvalidValue;
    }
#undef OCC_CASE
}

#ifndef CPM_RESIDENT_MODES_UNIT
size_t resident_smem_limit() { return 227 * 1024 - 4096; }

// 1: the 256-thread variant (two CTAs per SM), when its shared state fits
// half an SM; 0: the 512-thread variant.
int resident_variant(int64_t n_padded, int n_cells) {
    return res_layout(n_padded, n_cells, ResCfg<256>::CMAX).total <= resident_smem_limit() / 2 - 1024 ? 1 : 0;
}
size_t resident_smem_bytes(int64_t n_padded, int n_cells) {
    return resident_variant(n_padded, n_cells) ? res_layout(n_padded, n_cells, ResCfg<256>::CMAX).total
                                               : res_layout(n_padded, n_cells, ResCfg<512>::CMAX).total;
}
int resident_block(int variant) { return variant ? 256 : 512; }

cudaError_t prepare_resident_kernels() {
    cudaError_t e = prepare_resident_kernels_plain();
    return e == cudaSuccess ? prepare_resident_kernels_modes() : e;
}

cudaError_t launch_resident(int Dd, int NEd, int variant, int modes, SimDesc* d_sims, const RunPlan* d_plans,
                            int n_plans, int* d_next, const uint64_t* d_t3, size_t smem, int grid, cudaStream_t st) {
    return modes ? launch_resident_modes(Dd, NEd, variant, d_sims, d_plans, n_plans, d_next, d_t3, smem, grid, st)
                 : launch_resident_plain(Dd, NEd, variant, d_sims, d_plans, n_plans, d_next, d_t3, smem, grid, st);
}

cudaError_t resident_occupancy(int Dd, int NEd, int variant, int modes, size_t smem, int* blocks_per_sm) {
    return modes ? resident_occupancy_modes(Dd, NEd, variant, smem, blocks_per_sm)
                 : resident_occupancy_plain(Dd, NEd, variant, smem, blocks_per_sm);
}
#endif

#undef RES_MODES
#undef RES_VARIANT

}  // namespace cpmgpu
