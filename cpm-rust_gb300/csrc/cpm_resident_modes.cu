// Shared-memory resident sweep kernels for simulations with
// Metropolis-Hastings acceptance or the Act term (decide_modes): the kernels
// of cpm_resident_impl.cuh compiled in a unit of their own, in parallel with
// cpm_resident.cu.
#define CPM_RESIDENT_MODES_UNIT
#include "cpm_resident_impl.cuh"
