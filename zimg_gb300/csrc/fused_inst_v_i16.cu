// Instantiations of the fused streaming kernel for H_FIRST=false, U16, int32 sums.
#include "fused_inst.cuh"

ZG_FUSED_INSTANCE(v_i16, false, true, true)
