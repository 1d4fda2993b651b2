// Tiled sweep kernels for lattices with an odd periodic side (a third site
// colour for the last coordinate of each odd axis): the kernels of
// cpm_tiled.cu compiled in a unit of their own, in parallel with it.
#define CPM_TILED_ODD_UNIT
#include "cpm_tiled.cu"
