// Instantiations of the fused streaming kernel for H_FIRST=true, U16=true.
#include "fused_inst.cuh"

ZG_FUSED_INSTANCE(h_u16, true, true, false)
