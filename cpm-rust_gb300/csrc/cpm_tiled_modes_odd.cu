// Tiled sweep kernels for simulations with Metropolis-Hastings acceptance or
// the Act term on lattices with an odd periodic side: the kernels of
// cpm_tiled_impl.cuh compiled in a unit of their own.
#define CPM_TILED_MODES_UNIT
#define CPM_TILED_ODD_UNIT
#include "cpm_tiled_impl.cuh"
