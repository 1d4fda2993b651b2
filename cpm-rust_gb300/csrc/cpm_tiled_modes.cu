// Tiled sweep kernels for simulations with Metropolis-Hastings acceptance or
// the Act term, lattices with even (or fixed) sides: the kernels of
// cpm_tiled_impl.cuh compiled in a unit of their own, in parallel with the
// Metropolis units.
#define CPM_TILED_MODES_UNIT
#include "cpm_tiled_impl.cuh"
