// Instantiations of the fused streaming kernel for H_FIRST=true, U16=false.
#include "fused_inst.cuh"

ZG_FUSED_INSTANCE(h_f32, true, false, false)
