// sm_103a kernels of the GB300 Cellular Potts engine.
//
// sweep_kernel — the hot loop (reference: monte_carlo::run_mcs,
//   crates/cpm-core/src/monte_carlo.rs:327-357, wrapped by the run window of
//   output.rs:434-468). One CTA owns one simulation for its whole run plan:
//   every MCS is a random permutation of checkerboard colour passes; the
//   sites of one colour are pairwise >= 2 apart (Chebyshev, periodic wrap
//   included), so no attempt in a pass reads a site another attempt of the
//   same pass writes. What still couples attempts of one pass is the
//   per-cell volume and interface (global per cell). Those are resolved in
//   rounds: every pending candidate registers a 64-bit key (round tag,
//   per-pass random priority, class index) on both of its cells with a
//   shared-memory atomicMin, and a candidate that holds the minimum on both
//   cells is decided with the exact current V/I and committed. The pass is
//   therefore equivalent to applying its candidates one at a time in a
//   fixed order, each seeing exact state.
// evaluate_moves_kernel — per-move parity harness: decides a list of
//   (target, copy direction, u) on a frozen state with the same device
//   functions the sweep uses.
// recount_kernel / energy — exact recounts for the recount check and samples.
// table3d_kernel — generates the 2^26-bit 3D simple-point table on the
//   device from the bitmask flood fill (simple_point.rs:242-276).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include "cpm_common.h"
#include "cpm_device.cuh"
#include "cpm_kernels.h"

namespace cpmgpu {

constexpr int SWEEP_BLOCK = 512;
constexpr int SITES_PER_THREAD = 64;  // one u64 pending mask per thread per sub-batch

// ------------------------------------------------------------------------
// Colour classes. Axis d has 1, 2 or 3 colours: parity colours 0/1 cover
// coordinates [0, lim_d) with step 2; colour 2 (odd periodic axes only) is
// the single coordinate dims_d - 1, so same-colour sites never touch across
// the periodic seam.
// ------------------------------------------------------------------------
struct PassInfo {
    int cnt[3];
    int base[3];
    int step[3];
    int n;
};

__device__ __forceinline__ void make_pass(const SimDesc& s, int color, PassInfo& p) {
    int c = color;
    p.n = 1;
    for (int d = s.D - 1; d >= 0; --d) {  // last axis is the fastest colour digit
        const int cd = c % s.ncol[d];
        c /= s.ncol[d];
        if (cd == 2) { p.base[d] = s.dims[d] - 1; p.step[d] = 0; p.cnt[d] = 1; }
        else { p.base[d] = cd; p.step[d] = 2; p.cnt[d] = s.lim[d] > cd ? (s.lim[d] - cd + 1) / 2 : 0; }
        p.n *= p.cnt[d];
    }
    for (int d = s.D; d < 3; ++d) { p.cnt[d] = 1; p.base[d] = 0; p.step[d] = 0; }
}

template <int D>
__device__ __forceinline__ int site_of(const SimDesc& s, const PassInfo& p, int idx, int* x) {
    int f = 0;
#pragma unroll
    for (int d = D - 1; d >= 0; --d) {
        const int i = idx % p.cnt[d];
        idx /= p.cnt[d];
        x[d] = p.base[d] + p.step[d] * i;
        f += (x[d] + 1) * (int)s.strides[d];
    }
    return f;
}

__device__ __forceinline__ unsigned long long make_key(uint32_t tag, uint32_t pass_key, uint32_t idx) {
    const uint32_t prio = mix32(idx * 0x9E3779B9u ^ pass_key) >> 6;  // 26 bits
    return ((unsigned long long)tag << 48) | ((unsigned long long)prio << 22) | (unsigned long long)idx;
}

// ------------------------------------------------------------------------
// Block reduction of doubles in a fixed order (deterministic).
// ------------------------------------------------------------------------
template <int BLOCK>
__device__ double block_sum(double v, double* scratch) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < BLOCK / 32; ++w) t += scratch[w];
        scratch[0] = t;
    }
    __syncthreads();
    t = scratch[0];
    __syncthreads();
    return t;
}

// Global energy of the current state (energy.rs:104-113, 203-212, 266-308):
// each unordered neighbour pair of different cells contributes J once.
template <int D, int NE, int BLOCK>
__device__ double cta_energy(const SimDesc& s, double* scratch) {
    const uint32_t* sig = s.sigma;
    const int nt1 = s.n_types + 1;
    double ea = 0.0;
    for (int64_t q = threadIdx.x; q < s.n_sites; q += BLOCK) {
        int x[3];
        int64_t r = q;
        int f = 0;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
            x[d] = (int)(r % s.dims[d]);
            r /= s.dims[d];
            f += (x[d] + 1) * (int)s.strides[d];
        }
        const uint32_t c = sig[f];
        const int ci = s.adh_of[c];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const bool pos = (s.energy_pos_mask >> k) & 1u;
            bool count = pos;
            if (!pos && !s.periodic) {  // fixed boundary: bonds to the wall are never deduplicated
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const int y = x[d] + s.energy_vec[k][d];
                    if (y < 0 || y >= s.dims[d]) count = true;
                }
            }
            if (!count) continue;
            const uint32_t n = sig[f + (int)s.energy_off[k]];
            if (n != c) ea += s.J[ci * nt1 + s.adh_of[n]];
        }
    }
    double ev = 0.0, ei = 0.0;
    for (int id = 1 + threadIdx.x; id <= s.n_cells; id += BLOCK) {
        const int ty = s.adh_of[id] - 1;
        ev += quad_term(s.lambda_v[ty], s.target_v[ty], (double)s.volume[id]);
        ei += quad_term(s.lambda_i[ty], s.target_i[ty], (double)s.interface[id]);
    }
    ev = block_sum<BLOCK>(ev, scratch);
    ei = block_sum<BLOCK>(ei, scratch);
    ea = block_sum<BLOCK>(ea, scratch);
    return (ev + ei) + ea;
}

// ------------------------------------------------------------------------
// One colour pass of one MCS for the simulation owned by this CTA.
// ------------------------------------------------------------------------
struct Counters {
    unsigned long long attempts, nonnull, topo_reject, guard_reject, evaluated, accepted;
};

template <int D, int NE, int BLOCK>
__device__ void color_pass(const SimDesc& s, const PassInfo& p, uint64_t mcs, uint32_t pass_key,
                           unsigned long long* slots, const uint64_t* t3, uint32_t& tag, Counters& ct,
                           unsigned long long& rounds) {
    uint32_t* sig = s.sigma;
    const uint16_t* adh_of = s.adh_of;
    uint32_t* volume = s.volume;
    uint32_t* interface = s.interface;
    const int tid = threadIdx.x;
    for (int sb = 0; sb < p.n; sb += BLOCK * SITES_PER_THREAD) {
        // ---- build: early-out and connectivity, both functions of sigma only
        unsigned long long pend = 0, kb0 = 0, kb1 = 0, kb2 = 0;
        for (int i = 0; i < SITES_PER_THREAD; ++i) {
            const int idx = sb + tid + i * BLOCK;
            if (idx >= p.n) break;
            int x[3];
            const int t = site_of<D>(s, p, idx, x);
            const uint32_t L = sig[t];
            ct.attempts++;
            // every copy neighbour holds the target's cell: null whatever the
            // copy direction, so the draw (a counter, not a stream) is skipped
            if (copy_uniform(s, sig, t, L)) continue;
            const uint4 r = site_draw(s.seed, mcs, (uint32_t)t);
            const int k = (int)(((unsigned long long)r.x * (unsigned)s.n_copy) >> 32);
            const uint32_t G = sig[t + (int)s.copy_off[k]];
            if (L == G) continue;  // early-out (monte_carlo.rs:60-64)
            ct.nonnull++;
            if (!s.no_connectivity && !preserves_topology<D, uint32_t>(s, sig, t, L, s.table2d, t3)) {
                ct.topo_reject++;
                continue;
            }
            pend |= 1ull << i;
            kb0 |= (unsigned long long)(k & 1) << i;
            kb1 |= (unsigned long long)((k >> 1) & 1) << i;
            kb2 |= (unsigned long long)((k >> 2) & 1) << i;
        }
        // ---- rounds: lowest key on both cells decides with exact V/I
        for (;;) {
            for (unsigned long long m = pend; m; m &= m - 1) {
                const int i = __ffsll((long long)m) - 1;
                const int idx = sb + tid + i * BLOCK;
                int x[3];
                const int t = site_of<D>(s, p, idx, x);
                const int k = (int)((kb0 >> i) & 1) | (int)(((kb1 >> i) & 1) << 1) | (int)(((kb2 >> i) & 1) << 2);
                const uint32_t L = sig[t];
                const uint32_t G = sig[t + (int)s.copy_off[k]];
                const unsigned long long key = make_key(tag, pass_key, (uint32_t)idx);
                if (L) atomicMin(&slots[L], key);
                if (G) atomicMin(&slots[G], key);
            }
            __syncthreads();
            for (unsigned long long m = pend; m; m &= m - 1) {
                const int i = __ffsll((long long)m) - 1;
                const int idx = sb + tid + i * BLOCK;
                int x[3];
                const int t = site_of<D>(s, p, idx, x);
                const int k = (int)((kb0 >> i) & 1) | (int)(((kb1 >> i) & 1) << 1) | (int)(((kb2 >> i) & 1) << 2);
                const uint32_t L = sig[t];
                const uint32_t G = sig[t + (int)s.copy_off[k]];
                const unsigned long long key = make_key(tag, pass_key, (uint32_t)idx);
                if ((L && slots[L] != key) || (G && slots[G] != key)) continue;
                pend &= ~(1ull << i);
                if (L != 0 && volume[L] <= s.min_cell_volume) { ct.guard_reject++; continue; }
                ct.evaluated++;
                int dl = 0, dg = 0;
                const PhiloxDraw draw{s.seed, mcs, (uint32_t)t};
                const bool acc = (s.acceptance || s.act)
                                     ? decide_modes_sweep<NE>(s, sig, adh_of, volume, interface, t, t + s.copy_off[k], L,
                                                              G, mcs, draw, dl, dg)
                                     : decide_move<NE, uint32_t>(s, sig, adh_of, volume, interface, t, L, G, draw, dl, dg);
                if (acc) {
                    commit_move<D, uint32_t>(s, sig, volume, interface, s.sum_pos, s.sum_outer, x, L, G, dl, dg);
                    if (s.act) s.birth[t] = (uint32_t)mcs;  // energy.rs:453-458
                    ct.accepted++;
                }
            }
            const int any = __syncthreads_or(pend != 0);
            rounds++;
            if (!any) break;
            if (--tag == 0) {  // key space exhausted: clear the slots and restart the tags
                for (int c = tid; c <= s.n_cells; c += BLOCK) slots[c] = ~0ull;
                __syncthreads();
                tag = 0xFFFFu;
            }
        }
        if (--tag == 0) {
            for (int c = tid; c <= s.n_cells; c += BLOCK) slots[c] = ~0ull;
            __syncthreads();
            tag = 0xFFFFu;
        }
    }
}

template <int D, int NE, int BLOCK>
__device__ void one_mcs(const SimDesc& s, uint64_t mcs, unsigned long long* slots, const uint64_t* t3, int* perm,
                        PassInfo* pinfo, Counters& ct, unsigned long long& rounds) {
    if (threadIdx.x == 0) {
        // random colour order for this MCS (Fisher-Yates on Philox draws)
        const int nc = s.n_colors;
        for (int c = 0; c < nc; ++c) perm[c] = c;
        for (int c = nc - 1; c > 0; --c) {
            const uint4 r = aux_draw(s.seed, mcs, TAG_ORDER, (uint32_t)c, 0u);
            const int j = (int)(((unsigned long long)r.x * (unsigned)(c + 1)) >> 32);
            const int tmp = perm[c]; perm[c] = perm[j]; perm[j] = tmp;
        }
    }
    __syncthreads();
    for (int pi = 0; pi < s.n_colors; ++pi) {
        if (threadIdx.x == 0) make_pass(s, perm[pi], *pinfo);
        for (int c = threadIdx.x; c <= s.n_cells; c += BLOCK) slots[c] = ~0ull;
        __syncthreads();
        const PassInfo p = *pinfo;
        const uint32_t pass_key = aux_draw(s.seed, mcs, TAG_PASS, (uint32_t)pi, 0u).x;
        uint32_t tag = 0xFFFFu;
        color_pass<D, NE, BLOCK>(s, p, mcs, pass_key, slots, t3, tag, ct, rounds);
        __syncthreads();
    }
}

template <int D, int NE, int BLOCK>
__global__ void __launch_bounds__(BLOCK) sweep_kernel(SimDesc* sims, const RunPlan* plans, int n_plans,
                                                      int* next_plan, const uint64_t* t3, int slots_in_smem) {
    extern __shared__ unsigned long long dyn[];
    __shared__ SimDesc sd;
    __shared__ int s_plan;
    __shared__ int perm[27];
    __shared__ PassInfo pinfo;
    __shared__ double scratch[BLOCK / 32];
    __shared__ unsigned long long sstat[8];
    for (;;) {
        if (threadIdx.x == 0) s_plan = atomicAdd(next_plan, 1);
        __syncthreads();
        const int pl = s_plan;
        __syncthreads();
        if (pl >= n_plans) return;
        const RunPlan plan = plans[pl];
        if (threadIdx.x == 0) sd = sims[plan.sim];
        if (threadIdx.x < 8) sstat[threadIdx.x] = 0;
        __syncthreads();
        unsigned long long* slots = slots_in_smem ? dyn : sd.slots;
        Counters ct = {0, 0, 0, 0, 0, 0};
        unsigned long long rounds = 0;
        uint64_t mcs = sd.mcs;
        // burn-in (output.rs:441-454)
        uint64_t burned = 0;
        int e_idx = 0;
        while (burned < plan.burn_in) {
            const uint64_t chunk = plan.interval < plan.burn_in - burned ? plan.interval : plan.burn_in - burned;
            for (uint64_t m = 0; m < chunk; ++m, ++mcs) one_mcs<D, NE, BLOCK>(sd, mcs, slots, t3, perm, &pinfo, ct, rounds);
            burned += chunk;
            if (burned >= plan.energy_sample_start) {
                const double e = cta_energy<D, NE, BLOCK>(sd, scratch);
                if (threadIdx.x == 0 && sd.energy_out) sd.energy_out[e_idx] = e;
                ++e_idx;
            }
        }
        // readout (output.rs:463-468)
        for (int smp = 0; smp < plan.n_samples; ++smp) {
            for (uint64_t m = 0; m < plan.interval; ++m, ++mcs) one_mcs<D, NE, BLOCK>(sd, mcs, slots, t3, perm, &pinfo, ct, rounds);
            const double e = cta_energy<D, NE, BLOCK>(sd, scratch);
            if (threadIdx.x == 0 && sd.energy_out) sd.energy_out[e_idx + smp] = e;
            if (plan.write_samples) {
                const int n1 = sd.n_cells + 1;
                for (int id = threadIdx.x; id < n1; id += BLOCK) {
                    sd.sample_volume[(int64_t)smp * n1 + id] = sd.volume[id];
                    sd.sample_interface[(int64_t)smp * n1 + id] = sd.interface[id];
                    for (int d = 0; d < D; ++d) sd.sample_sum_pos[((int64_t)smp * n1 + id) * D + d] = sd.sum_pos[(int64_t)id * D + d];
                    for (int d = 0; d < D * D; ++d)
                        sd.sample_sum_outer[((int64_t)smp * n1 + id) * D * D + d] = sd.sum_outer[(int64_t)id * D * D + d];
                }
            }
            if (plan.write_lattice && sd.sample_lattice) {
                for (int64_t q = threadIdx.x; q < sd.n_sites; q += BLOCK) {
                    int64_t r = q;
                    int f = 0;
#pragma unroll
                    for (int d = D - 1; d >= 0; --d) {
                        f += ((int)(r % sd.dims[d]) + 1) * (int)sd.strides[d];
                        r /= sd.dims[d];
                    }
                    sd.sample_lattice[(int64_t)smp * sd.n_sites + q] = sd.sigma[f];
                }
            }
            __syncthreads();
        }
        // flush statistics
        atomicAdd(&sstat[CPM_STAT_ATTEMPTS], ct.attempts);
        atomicAdd(&sstat[CPM_STAT_NONNULL], ct.nonnull);
        atomicAdd(&sstat[CPM_STAT_TOPO_REJECT], ct.topo_reject);
        atomicAdd(&sstat[CPM_STAT_GUARD_REJECT], ct.guard_reject);
        atomicAdd(&sstat[CPM_STAT_EVALUATED], ct.evaluated);
        atomicAdd(&sstat[CPM_STAT_ACCEPTED], ct.accepted);
        __syncthreads();
        if (threadIdx.x < 6) atomicAdd(&sd.stats[threadIdx.x], sstat[threadIdx.x]);
        if (threadIdx.x == 0) {
            atomicAdd(&sd.stats[CPM_STAT_ROUNDS], rounds);
            atomicAdd(&sd.stats[CPM_STAT_PASSES], (unsigned long long)(mcs - sd.mcs) * sd.n_colors);
            sims[plan.sim].mcs = mcs;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------
// Per-move parity harness.
// ------------------------------------------------------------------------
template <int D, int NE>
__global__ void evaluate_moves_kernel(const SimDesc* simp, int64_t n, const int64_t* target, const int32_t* kdir,
                                      const double* u, MoveOut* out, const uint64_t* t3) {
    const SimDesc& s = *simp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        MoveOut o;
        o.target_flat = target[i];
        const int t = (int)target[i];
        o.source_flat = t + s.copy_off[kdir[i]];
        o.losing = s.sigma[t];
        o.gaining = s.sigma[o.source_flat];
        o.null_move = o.losing == o.gaining;
        o.topology_ok = 0; o.volume_guard_ok = 0; o.evaluated = 0;
        o.delta_i_losing = 0; o.delta_i_gaining = 0; o.delta_h = 0.0; o.accepted = 0; o.accepted_sweep = 0;
        if (!o.null_move) {
            o.topology_ok = preserves_topology<D, uint32_t>(s, s.sigma, t, o.losing, s.table2d, t3);
            if (o.topology_ok) {
                o.volume_guard_ok = !(o.losing != 0 && s.volume[o.losing] <= s.min_cell_volume);
                if (o.volume_guard_ok && (s.acceptance || s.act)) {
                    o.evaluated = 1;
                    int dl = 0, dg = 0;
                    double dh = 0.0;
                    o.accepted = decide_modes<NE>(s, s.sigma, s.adh_of, s.volume, s.interface, t, o.source_flat, o.losing,
                                                  o.gaining, s.mcs, GivenDraw{u[i]}, dl, dg, dh);
                    // the sweeps' decision (decide_modes_sweep: the float
                    // bracket when the Act delta is zero) on the same u
                    int dl2 = 0, dg2 = 0;
                    o.accepted_sweep = decide_modes_sweep<NE>(s, s.sigma, s.adh_of, s.volume, s.interface, t,
                                                              o.source_flat, o.losing, o.gaining, s.mcs,
                                                              GivenDraw{u[i]}, dl2, dg2);
                    o.delta_i_losing = dl;
                    o.delta_i_gaining = dg;
                    o.delta_h = dh;
                } else if (o.volume_guard_ok) {
                    o.evaluated = 1;
                    const DeltaOut d = delta_h<NE, uint32_t>(s, s.sigma, s.adh_of, s.volume, s.interface, t, o.losing, o.gaining);
                    o.delta_i_losing = d.dl;
                    o.delta_i_gaining = d.dg;
                    o.delta_h = d.dh;
                    o.accepted = metropolis(d.dh, u[i]);
                    int dl = 0, dg = 0;
                    o.accepted_sweep = decide_move<NE, uint32_t>(s, s.sigma, s.adh_of, s.volume, s.interface, t, o.losing,
                                                                 o.gaining, GivenDraw{u[i]}, dl, dg);
                }
            }
        }
        out[i] = o;
    }
}

// Applies a list of moves in order with the sweep's commit (single thread):
// the harness for the commit bookkeeping (dynamics.rs:23-183).
template <int D, int NE>
__global__ void commit_moves_kernel(const SimDesc* simp, int64_t n, const int64_t* target, const uint32_t* gaining) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const SimDesc& s = *simp;
    for (int64_t i = 0; i < n; ++i) {
        const int t = (int)target[i];
        const uint32_t L = s.sigma[t], G = gaining[i];
        const DeltaOut d = delta_h<NE, uint32_t>(s, s.sigma, s.adh_of, s.volume, s.interface, t, L, G);
        int x[3];
        coords_of<D>(s, t, x);
        commit_move<D, uint32_t>(s, s.sigma, s.volume, s.interface, s.sum_pos, s.sum_outer, x, L, G, d.dl, d.dg);
        if (s.act) s.birth[t] = (uint32_t)s.mcs;
    }
}

// Exact recount of V and I from sigma (checker.rs:36-83).
template <int D, int NE>
__global__ void recount_kernel(const SimDesc* simp, uint32_t* vol, uint32_t* itf) {
    const SimDesc& s = *simp;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < s.n_sites; q += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = q;
        int f = 0;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
            f += ((int)(r % s.dims[d]) + 1) * (int)s.strides[d];
            r /= s.dims[d];
        }
        const uint32_t c = s.sigma[f];
        if (!c) continue;
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < NE; ++k) cnt += s.sigma[f + (int)s.energy_off[k]] != c;
        atomicAdd(&vol[c], 1u);
        atomicAdd(&itf[c], (unsigned)cnt);
    }
}

template <int D, int NE>
__global__ void energy_kernel(const SimDesc* simp, double* out) {
    __shared__ double scratch[256 / 32];
    const double e = cta_energy<D, NE, 256>(*simp, scratch);
    if (threadIdx.x == 0) *out = e;
}

// One readout sample of a simulation whose state lives in HBM (the tiled
// path): V, I and the position sums into sample `smp`, and optionally the
// unpadded lattice.
template <int D>
__global__ void sample_kernel(const SimDesc* simp, int smp, int write_lattice) {
    const SimDesc& s = *simp;
    const int64_t n1 = s.n_cells + 1;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < n1; id += stride) {
        s.sample_volume[smp * n1 + id] = __ldcg(s.volume + id);
        s.sample_interface[smp * n1 + id] = __ldcg(s.interface + id);
        for (int d = 0; d < D; ++d)
            s.sample_sum_pos[(smp * n1 + id) * D + d] = __ldcg((const long long*)s.sum_pos + id * D + d);
        for (int d = 0; d < D * D; ++d)
            s.sample_sum_outer[(smp * n1 + id) * D * D + d] = __ldcg((const long long*)s.sum_outer + id * D * D + d);
    }
    if (write_lattice && s.sample_lattice) {
        for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < s.n_sites; q += stride) {
            int64_t r = q, f = 0;
            for (int d = D - 1; d >= 0; --d) {
                f += (r % s.dims[d] + 1) * s.strides[d];
                r /= s.dims[d];
            }
            s.sample_lattice[(int64_t)smp * s.n_sites + q] = __ldcg(s.sigma + f);
        }
    }
}

// 3D simple-point table: bit p set iff pattern p is simple (FastChecker).
__global__ void table3d_kernel(uint64_t* words, const uint32_t* face_adj, const uint32_t* full_adj,
                               uint32_t origin_face_mask) {
    __shared__ uint32_t fa[26], fu[26];
    if (threadIdx.x < 26) { fa[threadIdx.x] = face_adj[threadIdx.x]; fu[threadIdx.x] = full_adj[threadIdx.x]; }
    __syncthreads();
    const uint32_t full_mask = (1u << 26) - 1;
    const uint32_t nw = (1u << 26) / 64;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
        unsigned long long bits = 0;
        for (uint32_t b = 0; b < 64; ++b) {
            const uint32_t obj = w * 64 + b;
            const uint32_t cm = (~obj) & full_mask;
            // background: exactly one component under full adjacency
            int comps = 0;
            uint32_t rem = cm;
            while (rem && comps < 2) {
                uint32_t c = 1u << (__ffs(rem) - 1);
                for (;;) {
                    uint32_t nc = c;
                    for (uint32_t m = c; m; m &= m - 1) nc |= fu[__ffs(m) - 1] & cm;
                    if (nc == c) break;
                    c = nc;
                }
                rem &= ~c;
                ++comps;
            }
            if (comps != 1) continue;
            // object: exactly one face-component touching the origin
            int touching = 0;
            rem = obj;
            while (rem) {
                uint32_t c = 1u << (__ffs(rem) - 1);
                for (;;) {
                    uint32_t nc = c;
                    for (uint32_t m = c; m; m &= m - 1) nc |= fa[__ffs(m) - 1] & obj;
                    if (nc == c) break;
                    c = nc;
                }
                rem &= ~c;
                if (c & origin_face_mask) ++touching;
            }
            if (touching == 1) bits |= 1ull << b;
        }
        words[w] = bits;
    }
}

// ------------------------------------------------------------------------
// Host-side launchers.
// ------------------------------------------------------------------------
static int energy_index(int D, int NE) {
    if (D == 2 && NE == 4) return 0;
    if (D == 2 && NE == 8) return 1;
    if (D == 3 && NE == 6) return 2;
    if (D == 3 && NE == 18) return 3;
    if (D == 3 && NE == 26) return 4;
    return -1;
}

#define CPM_DISPATCH(D_, NE_, ...)                                   \
    switch (energy_index(D_, NE_)) {                                   \
        case 0: { constexpr int D = 2, NE = 4; __VA_ARGS__; break; }          \
        case 1: { constexpr int D = 2, NE = 8; __VA_ARGS__; break; }          \
        case 2: { constexpr int D = 3, NE = 6; __VA_ARGS__; break; }          \
        case 3: { constexpr int D = 3, NE = 18; __VA_ARGS__; break; }         \
        case 4: { constexpr int D = 3, NE = 26; __VA_ARGS__; break; }         \
        default: return cudaErrorInvalidValue;                         \
    }

size_t sweep_smem_bytes(int max_cells) { return (size_t)(max_cells + 1) * sizeof(unsigned long long); }

int sweep_max_smem_cells() { return (200 * 1024) / 8 - 2; }

cudaError_t launch_sweep(int Dd, int NEd, SimDesc* d_sims, const RunPlan* d_plans, int n_plans, int* d_next,
                         const uint64_t* d_t3, int max_cells, int grid, cudaStream_t st) {
    const int in_smem = max_cells <= sweep_max_smem_cells();
    const size_t smem = in_smem ? sweep_smem_bytes(max_cells) : 0;
    // the shared-memory limit is raised once per kernel and device (see
    // prepare_resident_kernels)
    static std::mutex mu;
    static bool done[64][5] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    CPM_DISPATCH(Dd, NEd, {
        auto k = sweep_kernel<D, NE, SWEEP_BLOCK>;
        {
            std::lock_guard<std::mutex> lk(mu);
            const int v = (D == 2 ? 0 : 2) + (NE == 8 || NE == 18 ? 1 : 0) + (NE == 26 ? 2 : 0);
            if (dev < 0 || dev >= 64 || !done[dev][v]) {
                cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
                if (e != cudaSuccess) return e;
                if (dev >= 0 && dev < 64) done[dev][v] = true;
            }
        }
        k<<<grid, SWEEP_BLOCK, smem, st>>>(d_sims, d_plans, n_plans, d_next, d_t3, in_smem);
    });
    return cudaGetLastError();
}

int sweep_block() { return SWEEP_BLOCK; }

cudaError_t launch_evaluate(int Dd, int NEd, const SimDesc* d_sim, int64_t n, const int64_t* d_t, const int32_t* d_k,
                            const double* d_u, MoveOut* d_out, const uint64_t* d_t3, cudaStream_t st) {
    const int grid = (int)((n + 255) / 256 > 4096 ? 4096 : (n + 255) / 256);
    CPM_DISPATCH(Dd, NEd, { evaluate_moves_kernel<D, NE><<<grid > 0 ? grid : 1, 256, 0, st>>>(d_sim, n, d_t, d_k, d_u, d_out, d_t3); });
    return cudaGetLastError();
}

cudaError_t launch_commit_moves(int Dd, int NEd, const SimDesc* d_sim, int64_t n, const int64_t* d_t, const uint32_t* d_g,
                                cudaStream_t st) {
    CPM_DISPATCH(Dd, NEd, { commit_moves_kernel<D, NE><<<1, 32, 0, st>>>(d_sim, n, d_t, d_g); });
    return cudaGetLastError();
}

cudaError_t launch_recount(int Dd, int NEd, const SimDesc* d_sim, int64_t n_sites, uint32_t* d_vol, uint32_t* d_itf,
                           cudaStream_t st) {
    int grid = (int)((n_sites + 255) / 256);
    if (grid > 8192) grid = 8192;
    if (grid < 1) grid = 1;
    CPM_DISPATCH(Dd, NEd, { recount_kernel<D, NE><<<grid, 256, 0, st>>>(d_sim, d_vol, d_itf); });
    return cudaGetLastError();
}

cudaError_t launch_energy(int Dd, int NEd, const SimDesc* d_sim, double* d_out, cudaStream_t st) {
    CPM_DISPATCH(Dd, NEd, { energy_kernel<D, NE><<<1, 256, 0, st>>>(d_sim, d_out); });
    return cudaGetLastError();
}

cudaError_t launch_sample(int Dd, const SimDesc* d_sim, int sample, int write_lattice, int64_t n_sites, cudaStream_t st) {
    int grid = (int)((n_sites + 255) / 256);
    if (grid > 4096) grid = 4096;
    if (grid < 1) grid = 1;
    if (Dd == 2) sample_kernel<2><<<grid, 256, 0, st>>>(d_sim, sample, write_lattice);
    else sample_kernel<3><<<grid, 256, 0, st>>>(d_sim, sample, write_lattice);
    return cudaGetLastError();
}

cudaError_t launch_table3d(uint64_t* d_words, const uint32_t* d_face, const uint32_t* d_full, uint32_t origin_mask,
                           cudaStream_t st) {
    table3d_kernel<<<1024, 256, 0, st>>>(d_words, d_face, d_full, origin_mask);
    return cudaGetLastError();
}

}  // namespace cpmgpu
