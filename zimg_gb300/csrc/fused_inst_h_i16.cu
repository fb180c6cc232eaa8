// Instantiations of the fused streaming kernel for H_FIRST=true, U16, int32 sums.
#include "fused_inst.cuh"

ZG_FUSED_INSTANCE(h_i16, true, true, true)
