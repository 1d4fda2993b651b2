// Tiled sweep kernels for lattices with an odd periodic side (a third site
// colour for the last coordinate of each odd axis): the kernels of
// cpm_tiled_impl.cuh compiled in a unit of their own, in parallel with
// cpm_tiled.cu.
#define CPM_TILED_ODD_UNIT
#include "cpm_tiled_impl.cuh"
