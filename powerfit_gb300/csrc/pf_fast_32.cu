// Fast-path kernels instantiated for 32^3 grids (the coarse grid of the learned proposal).
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_32() { return pf::FastSize<32>::table(); }
