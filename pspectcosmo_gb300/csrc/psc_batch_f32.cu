// Batched passes over several configurations (one launch per pass), FP32 instantiation.
#include "psc_batch.cuh"
PSC_DEFINE_BATCH_ENTRY(float, f32)
