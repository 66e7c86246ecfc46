// Fast-path kernels instantiated for 128^3 grids.
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_128() { return pf::FastSize<128>::table(); }
