// Fast-path kernels instantiated for 160^3 grids.
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_160() { return pf::FastSize<160>::table(); }
