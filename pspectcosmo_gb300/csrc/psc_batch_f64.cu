// Batched passes over several configurations (one launch per pass), FP64 instantiation.
#include "psc_batch.cuh"
PSC_DEFINE_BATCH_ENTRY(double, f64)
