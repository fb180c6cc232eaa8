// Instantiations of the fused streaming kernel for H_FIRST=false, U16=true.
#include "fused_inst.cuh"

ZG_FUSED_INSTANCE(v_u16, false, true, false)
