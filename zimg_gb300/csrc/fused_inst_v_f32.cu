// Instantiations of the fused streaming kernel for H_FIRST=false, U16=false.
#include "fused_inst.cuh"

ZG_FUSED_INSTANCE(v_f32, false, false, false)
