// Fast-path kernels instantiated for 64^3 grids.
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_64() { return pf::FastSize<64>::table(); }
