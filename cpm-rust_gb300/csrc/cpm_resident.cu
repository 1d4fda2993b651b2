// Shared-memory resident sweep kernels (Metropolis acceptance, no Act term)
// and the resident entry points shared with cpm_resident_modes.cu: the
// kernel source is cpm_resident_impl.cuh.
#include "cpm_resident_impl.cuh"
