// Register-engine passes, FP64 instantiation.
#include "psc_reg_impl.cuh"
PSC_DEFINE_REG_ENTRY(double, f64)
