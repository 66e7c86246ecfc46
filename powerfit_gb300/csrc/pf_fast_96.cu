// Fast-path kernels instantiated for 96^3 grids.
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_96() { return pf::FastSize<96>::table(); }
