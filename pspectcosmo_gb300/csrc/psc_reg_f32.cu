// Register-engine passes, FP32 instantiation.
#include "psc_reg_impl.cuh"
PSC_DEFINE_REG_ENTRY(float, f32)
