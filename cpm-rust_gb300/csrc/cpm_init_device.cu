// Initial state on the device: explicit-placement validation
// (initialization.rs:61-137) and the derived state of a fresh lattice
// (initialization.rs:396-436, without the contact graph, which the device
// readouts build per sample).
//
// Validation answers the three lattice questions of place_explicit in one
// upload and a few launches: the first site (in lattice order) whose id
// exceeds the cell count, the lowest cell id with no site, and the lowest
// cell id whose sites form more than one component under the connectivity
// neighbourhood (von Neumann, wrapping on periodic axes). Components come
// from a lock-free union-find over the sites (a root is the lowest site
// index of its component; links go from the larger root to the smaller by
// compare-and-swap, so every find walks to strictly lower indices and ends).
// The host turns the answers into the reference's messages in its order.
//
// The derived state is a sum over sites, so atomics give the exact integers
// the host loop gives, in any order: volume, interface (energy neighbours of
// another owner, halo included), and the position sums of interior
// coordinates.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cpm_common.h"
#include "cpm_kernels.h"

namespace cpmgpu {
namespace {

constexpr int IB = 256;

__global__ void range_volume_kernel(const uint32_t* lat, int64_t n_sites, uint32_t n_cells,
                                    unsigned long long* first_bad, uint32_t* volume) {
    for (int64_t i = blockIdx.x * (int64_t)IB + threadIdx.x; i < n_sites; i += (int64_t)gridDim.x * IB) {
        const uint32_t v = lat[i];
        if (v > n_cells) atomicMin(first_bad, (unsigned long long)i);
        else if (v) atomicAdd(volume + v, 1u);
    }
}

__global__ void lowest_zero_kernel(const uint32_t* volume, uint32_t n_cells, uint32_t* out) {
    for (uint32_t id = 1 + blockIdx.x * IB + threadIdx.x; id <= n_cells; id += gridDim.x * IB)
        if (volume[id] == 0) atomicMin(out, id);
}

__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x) {
    // L2 loads: links made by other SMs during the launch are seen
    uint32_t p = __ldcg(parent + x);
    while (p != x) {
        const uint32_t gp = __ldcg(parent + p);
        if (gp != p) parent[x] = gp;  // path halving: a lower ancestor, benign under races
        x = p;
        p = gp;
    }
    return x;
}

__device__ void uf_union(uint32_t* parent, uint32_t a, uint32_t b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t prev = atomicCAS(parent + hi, hi, lo);
        if (prev == hi) return;
        // hi was linked meanwhile: retry from its new parent (strictly lower)
        a = prev;
        b = lo;
    }
}

__global__ void uf_init_kernel(uint32_t* parent, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)IB + threadIdx.x; i < n; i += (int64_t)gridDim.x * IB)
        parent[i] = (uint32_t)i;
}

struct Grid3 {
    int D;
    int dims[3];
    int periodic;
};

// row-major interior index -> coordinates (last axis fastest)
__device__ __forceinline__ void coords_of(const Grid3& g, int64_t i, int* x) {
    for (int d = g.D - 1; d >= 0; --d) {
        x[d] = (int)(i % g.dims[d]);
        i /= g.dims[d];
    }
}

// Each site joins its same-cell neighbour one step up every axis (wrapping
// on a periodic lattice): every von Neumann pair once.
__global__ void uf_link_kernel(const uint32_t* lat, uint32_t* parent, Grid3 g, int64_t n_sites, uint32_t n_cells) {
    for (int64_t i = blockIdx.x * (int64_t)IB + threadIdx.x; i < n_sites; i += (int64_t)gridDim.x * IB) {
        const uint32_t v = lat[i];
        if (v == 0 || v > n_cells) continue;
        int x[3] = {0, 0, 0};
        coords_of(g, i, x);
        int64_t stride = 1;
        for (int d = g.D - 1; d >= 0; --d) {
            int64_t j = -1;
            if (x[d] + 1 < g.dims[d]) j = i + stride;
            else if (g.periodic && g.dims[d] > 1) j = i - (int64_t)(g.dims[d] - 1) * stride;
            if (j >= 0 && lat[j] == v) uf_union(parent, (uint32_t)i, (uint32_t)j);
            stride *= g.dims[d];
        }
    }
}

__global__ void uf_cell_root_kernel(const uint32_t* lat, uint32_t* parent, int64_t n_sites, uint32_t n_cells,
                                    uint32_t* cell_root) {
    for (int64_t i = blockIdx.x * (int64_t)IB + threadIdx.x; i < n_sites; i += (int64_t)gridDim.x * IB) {
        const uint32_t v = lat[i];
        if (v == 0 || v > n_cells) continue;
        atomicMin(cell_root + v, uf_find(parent, (uint32_t)i));
    }
}

__global__ void uf_split_kernel(const uint32_t* lat, uint32_t* parent, int64_t n_sites, uint32_t n_cells,
                                const uint32_t* cell_root, uint32_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)IB + threadIdx.x; i < n_sites; i += (int64_t)gridDim.x * IB) {
        const uint32_t v = lat[i];
        if (v == 0 || v > n_cells) continue;
        if (uf_find(parent, (uint32_t)i) != cell_root[v]) atomicMin(out, v);
    }
}

// Derived state of every simulation of a set (blockIdx.y = simulation): the
// sums over interior sites of initialization.rs:396-436. A warp whose 32
// sites all hold one cell (the usual case inside cells) adds its terms with
// one atomic per quantity; other sites add their own.
__device__ __forceinline__ long long warp_sum64(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void derive_kernel(const SimDesc* sims) {
    const SimDesc& s = sims[blockIdx.y];
    const int D = s.D;
    const int64_t n = s.n_sites;
    const int64_t step = (int64_t)gridDim.x * IB;
    // a uniform trip count over the block, so that every lane takes part in
    // the warp-wide match
    for (int64_t base = blockIdx.x * (int64_t)IB; base < n; base += step) {
        const int64_t i = base + threadIdx.x;
        int x[3] = {0, 0, 0};
        int64_t f = 0;
        uint32_t cell = 0;
        if (i < n) {
            int64_t r = i;
            for (int d = D - 1; d >= 0; --d) {
                x[d] = (int)(r % s.dims[d]);
                r /= s.dims[d];
            }
            for (int d = 0; d < D; ++d) f += (int64_t)(x[d] + 1) * s.strides[d];
            cell = s.sigma[f];
        }
        uint32_t itf = 0;
        if (cell)
            for (int k = 0; k < s.n_energy; ++k) itf += s.sigma[f + s.energy_off[k]] != cell;
        const unsigned peers = __match_any_sync(0xffffffffu, cell);
        if (peers == 0xffffffffu) {
            // one owner for the whole warp (uniform branch)
            if (cell == 0) continue;
            const uint32_t itf_w = __reduce_add_sync(0xffffffffu, itf);
            long long sp[3], so[9];
            for (int d = 0; d < D; ++d) sp[d] = warp_sum64((long long)x[d]);
            for (int d = 0; d < D; ++d)
                for (int e = 0; e < D; ++e) so[d * 3 + e] = warp_sum64((long long)x[d] * x[e]);
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(s.volume + cell, 32u);
                atomicAdd(s.interface + cell, itf_w);
                for (int d = 0; d < D; ++d)
                    atomicAdd((unsigned long long*)(s.sum_pos + (int64_t)cell * D + d), (unsigned long long)sp[d]);
                for (int d = 0; d < D; ++d)
                    for (int e = 0; e < D; ++e)
                        atomicAdd((unsigned long long*)(s.sum_outer + ((int64_t)cell * D + d) * D + e),
                                  (unsigned long long)so[d * 3 + e]);
            }
        } else if (cell) {
            atomicAdd(s.volume + cell, 1u);
            atomicAdd(s.interface + cell, itf);
            for (int d = 0; d < D; ++d)
                atomicAdd((unsigned long long*)(s.sum_pos + (int64_t)cell * D + d), (unsigned long long)(long long)x[d]);
            for (int d = 0; d < D; ++d)
                for (int e = 0; e < D; ++e)
                    atomicAdd((unsigned long long*)(s.sum_outer + ((int64_t)cell * D + d) * D + e),
                              (unsigned long long)((long long)x[d] * x[e]));
        }
    }
}

int grid_for(int64_t n) {
    const int64_t b = (n + IB - 1) / IB;
    return (int)(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

}  // namespace

cudaError_t launch_derive(const SimDesc* d_sims, int n_sims, int64_t max_sites, cudaStream_t st) {
    if (n_sims <= 0) return cudaSuccess;
    const int64_t b = (max_sites + IB - 1) / IB;
    const int gx = (int)(b < 1 ? 1 : (b > 1024 ? 1024 : b));
    for (int s0 = 0; s0 < n_sims; s0 += 65535) {
        const int ny = n_sims - s0 < 65535 ? n_sims - s0 : 65535;
        derive_kernel<<<dim3(gx, ny), IB, 0, st>>>(d_sims + s0);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t check_explicit_lattice(int D, const int64_t* dims, int periodic, const uint32_t* lattice, int64_t n_sites,
                                   uint32_t n_cells, ExplicitCheck* out) {
    out->first_bad_site = -1;
    out->zero_volume_id = 0;
    out->disconnected_id = 0;
    if (n_sites <= 0) return cudaSuccess;
    if (n_sites >= ((int64_t)1 << 32)) return cudaErrorInvalidValue;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    // one allocation: lattice, parents, volumes, cell roots, answers
    const size_t n1 = (size_t)n_cells + 1;
    const size_t b_lat = (size_t)n_sites * 4, b_par = (size_t)n_sites * 4, b_vol = n1 * 4, b_root = n1 * 4;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t total = up(b_lat) + up(b_par) + up(b_vol) + up(b_root) + 256;
    char* buf = nullptr;
    e = cudaMallocAsync((void**)&buf, total, st);
    if (e != cudaSuccess) {
        cudaStreamDestroy(st);
        return e;
    }
    uint32_t* d_lat = (uint32_t*)buf;
    uint32_t* d_par = (uint32_t*)(buf + up(b_lat));
    uint32_t* d_vol = (uint32_t*)(buf + up(b_lat) + up(b_par));
    uint32_t* d_root = (uint32_t*)(buf + up(b_lat) + up(b_par) + up(b_vol));
    unsigned long long* d_ans = (unsigned long long*)(buf + up(b_lat) + up(b_par) + up(b_vol) + up(b_root));
    uint32_t* d_zero = (uint32_t*)(d_ans + 1);
    uint32_t* d_split = d_zero + 1;
    Grid3 g{D, {1, 1, 1}, periodic};
    for (int d = 0; d < D; ++d) g.dims[d] = (int)dims[d];
    const int gs = grid_for(n_sites), gc = grid_for((int64_t)n1);
    struct Answers { unsigned long long bad; uint32_t zero, split; } h{};
    do {
        if ((e = cudaMemcpyAsync(d_lat, lattice, b_lat, cudaMemcpyHostToDevice, st))) break;
        if ((e = cudaMemsetAsync(d_vol, 0, b_vol, st))) break;
        if ((e = cudaMemsetAsync(d_root, 0xFF, b_root, st))) break;
        if ((e = cudaMemsetAsync(d_ans, 0xFF, 16, st))) break;
        range_volume_kernel<<<gs, IB, 0, st>>>(d_lat, n_sites, n_cells, d_ans, d_vol);
        lowest_zero_kernel<<<gc, IB, 0, st>>>(d_vol, n_cells, d_zero);
        uf_init_kernel<<<gs, IB, 0, st>>>(d_par, n_sites);
        uf_link_kernel<<<gs, IB, 0, st>>>(d_lat, d_par, g, n_sites, n_cells);
        uf_cell_root_kernel<<<gs, IB, 0, st>>>(d_lat, d_par, n_sites, n_cells, d_root);
        uf_split_kernel<<<gs, IB, 0, st>>>(d_lat, d_par, n_sites, n_cells, d_root, d_split);
        if ((e = cudaGetLastError())) break;
        if ((e = cudaMemcpyAsync(&h, d_ans, 16, cudaMemcpyDeviceToHost, st))) break;
        e = cudaStreamSynchronize(st);
    } while (false);
    const cudaError_t ef = cudaFreeAsync(buf, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (e == cudaSuccess) e = ef != cudaSuccess ? ef : es;
    if (e != cudaSuccess) return e;
    out->first_bad_site = h.bad == ~0ull ? -1 : (int64_t)h.bad;
    out->zero_volume_id = h.zero == 0xFFFFFFFFu ? 0u : h.zero;
    out->disconnected_id = h.split == 0xFFFFFFFFu ? 0u : h.split;
    return cudaSuccess;
}

}  // namespace cpmgpu
