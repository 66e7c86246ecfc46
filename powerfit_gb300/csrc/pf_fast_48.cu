// Fast-path kernels instantiated for 48^3 grids.
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_48() { return pf::FastSize<48>::table(); }
