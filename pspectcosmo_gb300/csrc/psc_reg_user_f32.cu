// Register-engine Z passes of the user models (model.h files compiled in), FP32 instantiation.
#include "psc_reg_impl.cuh"
PSC_DEFINE_REG_USER_ENTRY(float, f32)
