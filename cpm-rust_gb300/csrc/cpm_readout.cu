// Topology readouts of lattice snapshots on the device (sm_103a).
//
// Per sample the reference reads (output.rs:304-337):
//  * the contact graph (state.rs:127-157): for every unordered pair of
//    energy-neighbouring sites owned by different cells, one count on the
//    pair (min id, max id); a site pair is visited once, from the site with
//    the lower index, except against a fixed-boundary halo, which holds the
//    medium (0) and is counted from every interior site that sees it;
//  * the labelling (labelling.rs:70-154): the number of components of every
//    cell under the von Neumann stencil (cells with more than one are
//    "fragmented"), and the components of the medium under the full stencil
//    with their volumes and whether they touch a fixed boundary, in the order
//    a scan over the sites discovers them (ascending lowest site index).
//
// Here the contact counts go to a dense upper-triangular table per
// simulation (atomic adds), the components come from a lock-free union-find
// whose roots are the lowest site index of each component (a root is only
// ever linked below a smaller root), and every output stream is compacted in
// index order with a per-unit count pass and a prefix sum, so the host
// receives sorted lists and sorts nothing.
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include "cpm_common.h"
#include "cpm_kernels.h"

namespace {

constexpr int RO_BLOCK = 256;
constexpr int RO_PER_THREAD = 4;
constexpr int RO_UNIT = RO_BLOCK * RO_PER_THREAD;
constexpr int RO_WARPS = RO_BLOCK / 32;

// Largest item i with prefix[i] <= u (items own consecutive unit ranges).
__device__ __forceinline__ int item_of(const int64_t* prefix, int n_items, int64_t u) {
    int lo = 0, hi = n_items - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void coords_of(const ReadoutItem& it, uint32_t j, int x[3]) {
    if (it.D == 2) {
        x[0] = (int)(j / (uint32_t)it.dims[1]);
        x[1] = (int)(j - (uint32_t)x[0] * (uint32_t)it.dims[1]);
        x[2] = 0;
    } else {
        const uint32_t plane = (uint32_t)it.dims[1] * (uint32_t)it.dims[2];
        x[0] = (int)(j / plane);
        const uint32_t r = j - (uint32_t)x[0] * plane;
        x[1] = (int)(r / (uint32_t)it.dims[2]);
        x[2] = (int)(r - (uint32_t)x[1] * (uint32_t)it.dims[2]);
    }
}

// Interior index of x + o (wrapped on a periodic lattice); false when x + o
// lies in a fixed boundary's halo.
__device__ __forceinline__ bool neighbour_of(const ReadoutItem& it, const int x[3], int o0, int o1, int o2,
                                             uint32_t& k) {
    int y[3] = {x[0] + o0, x[1] + o1, x[2] + o2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d < it.D && (y[d] < 0 || y[d] >= it.dims[d])) {
            if (!it.periodic) return false;
            y[d] = y[d] < 0 ? y[d] + it.dims[d] : y[d] - it.dims[d];
        }
    }
    k = it.D == 2 ? (uint32_t)y[0] * (uint32_t)it.dims[1] + (uint32_t)y[1]
                  : ((uint32_t)y[0] * (uint32_t)it.dims[1] + (uint32_t)y[1]) * (uint32_t)it.dims[2] + (uint32_t)y[2];
    return true;
}

__device__ __forceinline__ bool on_surface(const ReadoutItem& it, const int x[3]) {
    bool s = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) s |= d < it.D && (x[d] == 0 || x[d] == it.dims[d] - 1);
    return s;
}

// Visits the offsets o in {-1,0,1}^D with 1..maxnz nonzero components; with
// `forward`, only those whose first nonzero component is positive (one of
// each pair o, -o).
template <class F>
__device__ __forceinline__ void for_offsets(int D, int maxnz, bool forward, F&& f) {
    const int r2 = D == 3 ? 1 : 0;
    for (int o0 = -1; o0 <= 1; ++o0)
        for (int o1 = -1; o1 <= 1; ++o1)
            for (int o2 = -r2; o2 <= r2; ++o2) {
                const int nz = (o0 != 0) + (o1 != 0) + (o2 != 0);
                if (nz == 0 || nz > maxnz) continue;
                if (forward && !(o0 > 0 || (o0 == 0 && (o1 > 0 || (o1 == 0 && o2 > 0))))) continue;
                f(o0, o1, o2);
            }
}

// Slot of the pair (a, b), a < b <= n, in the row-major upper triangle:
// row a holds b = a+1..n.
__device__ __forceinline__ uint64_t pair_slot(uint32_t n, uint32_t a, uint32_t b) {
    return (uint64_t)a * n - ((uint64_t)a * (a - 1ull) >> 1) + (b - a - 1u);
}

__device__ __forceinline__ uint64_t row_start(uint64_t n, uint64_t a) { return a * n - ((a * (a - 1ull)) >> 1); }

__device__ __forceinline__ void pair_of(uint32_t n, uint64_t e, uint32_t& a, uint32_t& b) {
    const double m = 2.0 * (double)n + 1.0;
    double g = 0.5 * (m - sqrt(m * m - 8.0 * (double)e));
    int64_t r = (int64_t)g;
    if (r < 0) r = 0;
    if (r > (int64_t)n - 1) r = (int64_t)n - 1;
    while (r + 1 <= (int64_t)n - 1 && row_start(n, (uint64_t)r + 1) <= e) ++r;
    while (r > 0 && row_start(n, (uint64_t)r) > e) --r;
    a = (uint32_t)r;
    b = (uint32_t)(e - row_start(n, (uint64_t)r)) + a + 1u;
}

// Root of v with path halving (in global or shared memory). Parents always
// point to lower indices, so every step lowers v and the walk ends; a stale
// read only yields an older ancestor, and a link (compare-and-swap) on a
// node that is no longer a root fails and returns its current parent.
__device__ __forceinline__ uint32_t find_root(uint32_t* p, uint32_t v) {
    for (;;) {
        const uint32_t par = p[v];
        if (par == v) return v;
        const uint32_t gp = p[par];
        if (gp == par) return par;
        p[v] = gp;  // v is not a root: no link can target it
        v = gp;
    }
}

// Links the trees of a and b, the larger root below the smaller. A failed
// compare-and-swap returns the root's new parent, which is lower, so each
// retry lowers one side and the loop ends.
__device__ __forceinline__ void unite(uint32_t* p, uint32_t a, uint32_t b) {
    uint32_t ra = find_root(p, a), rb = find_root(p, b);
    while (ra != rb) {
        if (ra > rb) {
            const uint32_t old = atomicCAS(p + ra, ra, rb);
            if (old == ra) return;
            ra = old;
        } else {
            const uint32_t old = atomicCAS(p + rb, rb, ra);
            if (old == rb) return;
            rb = old;
        }
    }
}

// Pass 0: medium words cleared, contact counts; a pair slot's first count
// also counts the slot in its unit of the pair stream.
__global__ void __launch_bounds__(RO_BLOCK) readout_contact_kernel(const ReadoutItem* items, int n_items,
                                                                   const int64_t* prefix, int64_t total,
                                                                   uint32_t* cnt) {
    for (int64_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int ii = item_of(prefix, n_items, u);
        const ReadoutItem it = items[ii];
        const int64_t u0 = prefix[ii], lu = u - u0;
        const uint32_t n = (uint32_t)it.n_cells;
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const int64_t j64 = lu * RO_UNIT + q * RO_BLOCK + threadIdx.x;
            if (j64 >= it.n_sites) break;
            const uint32_t j = (uint32_t)j64;
            it.aux[j] = 0u;
            const uint32_t a = it.lat[j];
            int x[3];
            coords_of(it, j, x);
            for_offsets(it.D, it.energy_maxnz, false, [&](int o0, int o1, int o2) {
                uint32_t k = 0, b = 0u;
                if (neighbour_of(it, x, o0, o1, o2, k)) {
                    if (k <= j) return;  // the pair is counted from the lower index
                    b = it.lat[k];
                }
                if (b == a) return;
                const uint32_t lo = min(a, b), hi = max(a, b);
                if (hi > n) return;  // not a cell id of this simulation
                const uint64_t e = pair_slot(n, lo, hi);
                if (atomicAdd(it.tri + e, 1u) == 0u) atomicAdd(cnt + 3 * (u0 + (int64_t)(e / RO_UNIT)), 1u);
            });
        }
    }
}

// Pass 1: the forest inside each unit (its sites are consecutive indices):
// every site joined with its same-owner neighbours (von Neumann for cells,
// the full stencil for the medium) that lie in the same unit, in shared
// memory; each site's parent becomes the lowest index of its unit-local
// component.
__global__ void __launch_bounds__(RO_BLOCK) readout_join_local_kernel(const ReadoutItem* items, int n_items,
                                                                      const int64_t* prefix, int64_t total) {
    __shared__ uint32_t s_lat[RO_UNIT];
    __shared__ uint32_t s_par[RO_UNIT];
    for (int64_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int ii = item_of(prefix, n_items, u);
        const ReadoutItem it = items[ii];
        const int64_t base64 = (u - prefix[ii]) * RO_UNIT;
        if (base64 >= it.n_sites) continue;  // block-uniform
        const uint32_t base = (uint32_t)base64;
        const int len = (int)((it.n_sites - base64) < RO_UNIT ? (it.n_sites - base64) : (int64_t)RO_UNIT);
        for (int l = threadIdx.x; l < RO_UNIT; l += RO_BLOCK) {
            s_par[l] = (uint32_t)l;
            s_lat[l] = l < len ? it.lat[base + l] : 0xFFFFFFFFu;
        }
        __syncthreads();
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const int l = q * RO_BLOCK + threadIdx.x;
            if (l >= len) break;
            const uint32_t j = base + (uint32_t)l;
            const uint32_t a = s_lat[l];
            int x[3];
            coords_of(it, j, x);
            for_offsets(it.D, a != 0u ? 1 : it.D, true, [&](int o0, int o1, int o2) {
                uint32_t k = 0;
                if (!neighbour_of(it, x, o0, o1, o2, k) || k == j || k < base || k - base >= (uint32_t)len) return;
                if (s_lat[k - base] == a) unite(s_par, (uint32_t)l, k - base);
            });
        }
        __syncthreads();
        for (int l = threadIdx.x; l < len; l += RO_BLOCK) it.parent[base + l] = base + find_root(s_par, (uint32_t)l);
        __syncthreads();
    }
}

// Pass 2: joins the same-owner neighbour pairs that cross units, on the
// global forest.
__global__ void __launch_bounds__(RO_BLOCK) readout_join_cross_kernel(const ReadoutItem* items, int n_items,
                                                                      const int64_t* prefix, int64_t total) {
    for (int64_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int ii = item_of(prefix, n_items, u);
        const ReadoutItem it = items[ii];
        const int64_t base64 = (u - prefix[ii]) * RO_UNIT;
        if (base64 >= it.n_sites) continue;
        const uint32_t base = (uint32_t)base64;
        const uint32_t len = (uint32_t)((it.n_sites - base64) < RO_UNIT ? (it.n_sites - base64) : (int64_t)RO_UNIT);
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const uint32_t l = (uint32_t)(q * RO_BLOCK + threadIdx.x);
            if (l >= len) break;
            const uint32_t j = base + l;
            const uint32_t a = it.lat[j];
            int x[3];
            coords_of(it, j, x);
            for_offsets(it.D, a != 0u ? 1 : it.D, true, [&](int o0, int o1, int o2) {
                uint32_t k = 0;
                if (!neighbour_of(it, x, o0, o1, o2, k) || (k >= base && k - base < len)) return;
                if (it.lat[k] == a) unite(it.parent, j, k);
            });
        }
    }
}

// Pass 3: roots (compressing the forest), component counts per cell (a
// cell's second root marks it fragmented and counts its id in the fragment
// stream), medium volumes and boundary contact per root, medium roots per
// unit of the medium stream.
__global__ void __launch_bounds__(RO_BLOCK) readout_roots_kernel(const ReadoutItem* items, int n_items,
                                                                 const int64_t* prefix, int64_t total,
                                                                 uint32_t* cnt) {
    __shared__ uint32_t s_roots;
    for (int64_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int ii = item_of(prefix, n_items, u);
        const ReadoutItem it = items[ii];
        const int64_t u0 = prefix[ii], lu = u - u0;
        if (threadIdx.x == 0) s_roots = 0u;
        __syncthreads();
        uint32_t my_roots = 0u;
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const int64_t j64 = lu * RO_UNIT + q * RO_BLOCK + threadIdx.x;
            bool med = false;
            uint32_t r = 0xFFFFFFFFu;
            if (j64 < it.n_sites) {
                const uint32_t j = (uint32_t)j64;
                r = find_root(it.parent, j);
                if (r != j) it.parent[j] = r;
                const uint32_t a = it.lat[j];
                if (a != 0u) {
                    if (r == j && a <= (uint32_t)it.n_cells && atomicAdd(it.ncomp + a, 1u) == 1u)
                        atomicAdd(cnt + 3 * (u0 + (int64_t)(a / RO_UNIT)) + 2, 1u);
                } else {
                    med = true;
                    if (r == j) ++my_roots;
                    if (!it.periodic) {
                        int x[3];
                        coords_of(it, j, x);
                        if (on_surface(it, x)) atomicOr(it.aux + r, 0x80000000u);
                    }
                }
            }
            // medium volumes: one add per root and warp
            const unsigned grp = __match_any_sync(0xFFFFFFFFu, med ? r : 0xFFFFFFFFu);
            if (med && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(it.aux + r, (uint32_t)__popc(grp));
        }
        if (my_roots) atomicAdd(&s_roots, my_roots);
        __syncthreads();
        if (threadIdx.x == 0 && s_roots) atomicAdd(cnt + 3 * u + 1, s_roots);
        __syncthreads();
    }
}

// Exclusive prefix sum of c over the block (all threads call it).
__device__ __forceinline__ uint32_t block_exclusive(uint32_t c, uint32_t* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = c;
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        const uint32_t t = lane < RO_WARPS ? sh[lane] : 0u;
        uint32_t s = t;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, d);
            if (lane >= d) s += y;
        }
        if (lane < RO_WARPS) sh[lane] = s - t;
    }
    __syncthreads();
    const uint32_t r = sh[w] + x - c;
    __syncthreads();
    return r;
}

// Pass 4: the three output streams in index order, each unit at its prefix
// offset; contact slots and component counts are reset to zero on the way.
__global__ void __launch_bounds__(RO_BLOCK) readout_emit_kernel(const ReadoutItem* items, int n_items,
                                                                const int64_t* prefix, int64_t total,
                                                                const uint64_t* off, uint32_t* pairs,
                                                                uint32_t* medium, uint32_t* frag) {
    __shared__ uint32_t sh[RO_WARPS];
    for (int64_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int ii = item_of(prefix, n_items, u);
        const ReadoutItem it = items[ii];
        const int64_t lu = u - prefix[ii];
        const int64_t base = lu * RO_UNIT + (int64_t)threadIdx.x * RO_PER_THREAD;
        const uint32_t n = (uint32_t)it.n_cells;
        // contact pairs
        uint32_t v[RO_PER_THREAD];
        uint32_t c = 0;
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const int64_t e = base + q;
            v[q] = e < it.tri_n ? it.tri[e] : 0u;
            c += v[q] != 0u;
        }
        uint64_t pos = off[3 * u] + block_exclusive(c, sh);
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            if (!v[q]) continue;
            const uint64_t e = (uint64_t)(base + q);
            uint32_t a, b;
            pair_of(n, e, a, b);
            pairs[3 * pos] = a;
            pairs[3 * pos + 1] = b;
            pairs[3 * pos + 2] = v[q];
            it.tri[e] = 0u;
            ++pos;
        }
        // medium components (roots in site order)
        uint32_t w[RO_PER_THREAD];
        uint32_t mf = 0;
        c = 0;
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const int64_t j = base + q;
            const bool root = j < it.n_sites && it.lat[j] == 0u && it.parent[j] == (uint32_t)j;
            w[q] = root ? it.aux[j] : 0u;
            if (root) { ++c; mf |= 1u << q; }
        }
        pos = off[3 * u + 1] + block_exclusive(c, sh);
        for (int q = 0; q < RO_PER_THREAD; ++q)
            if (mf & (1u << q)) medium[pos++] = w[q];
        // fragmented cells (ids in order)
        c = 0;
        uint32_t fl = 0;
        for (int q = 0; q < RO_PER_THREAD; ++q) {
            const int64_t id = base + q;
            if (id >= 1 && id <= (int64_t)n) {
                const uint32_t k = it.ncomp[id];
                if (k > 1u) { ++c; fl |= 1u << q; }
                if (k) it.ncomp[id] = 0u;
            }
        }
        pos = off[3 * u + 2] + block_exclusive(c, sh);
        for (int q = 0; q < RO_PER_THREAD; ++q)
            if (fl & (1u << q)) frag[pos++] = (uint32_t)(base + q);
    }
}

}  // namespace

namespace cpmgpu {

int readout_unit() { return RO_UNIT; }

cudaError_t launch_readout(int pass, const ReadoutItem* d_items, int n_items, const int64_t* d_prefix,
                           int64_t total_units, uint32_t* d_unit_cnt, const uint64_t* d_unit_off, uint32_t* d_pairs,
                           uint32_t* d_medium, uint32_t* d_frag, cudaStream_t st) {
    if (total_units <= 0 || n_items <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int grid = (int)std::min<int64_t>(total_units, (int64_t)sms * 8);
    switch (pass) {
        case 0:
            readout_contact_kernel<<<grid, RO_BLOCK, 0, st>>>(d_items, n_items, d_prefix, total_units, d_unit_cnt);
            break;
        case 1:
            readout_join_local_kernel<<<grid, RO_BLOCK, 0, st>>>(d_items, n_items, d_prefix, total_units);
            break;
        case 2:
            readout_join_cross_kernel<<<grid, RO_BLOCK, 0, st>>>(d_items, n_items, d_prefix, total_units);
            break;
        case 3:
            readout_roots_kernel<<<grid, RO_BLOCK, 0, st>>>(d_items, n_items, d_prefix, total_units, d_unit_cnt);
            break;
        case 4:
            readout_emit_kernel<<<grid, RO_BLOCK, 0, st>>>(d_items, n_items, d_prefix, total_units, d_unit_off,
                                                           d_pairs, d_medium, d_frag);
            break;
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace cpmgpu
