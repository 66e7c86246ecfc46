// Fast-path kernels instantiated for 192^3 grids (plane pass on a four-block cluster).
#include "pf_kernels_ct.cuh"

pf::FastLaunch pf_fast_table_192() { return pf::FastSize<192>::table(); }
