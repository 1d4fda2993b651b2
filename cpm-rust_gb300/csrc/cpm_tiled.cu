// Tiled sweep kernels for lattices with even (or fixed) sides: the kernels
// of cpm_tiled_impl.cuh, plus the shared host entry points (tile plan,
// shared-memory sizes, the dispatch between the even and odd-side units).
#include "cpm_tiled_impl.cuh"
