// psc_model.h — the model surface (model.h) in FP64 for host and device code: the two
// built-in models and the user models compiled from model.h files (psc_user_models.cuh,
// generated by model_adapter.py at build time). The per-site evaluation of the passes in
// the field precision is in psc_dev.cuh.
#pragma once

#include "../../include/psc.h"
#include "psc_user_models.cuh"

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace psc {

static_assert(kUserMaxFields == PSC_MAX_FIELDS && kUserMaxTerms == PSC_MAX_TERMS, "model limits");

__host__ __device__ inline bool model_is_user(int model) {
    return model >= PSC_MODEL_USER && model < PSC_MODEL_USER + kUserModels;
}
__host__ __device__ inline bool model_known(int model) {
    return model == PSC_MODEL_PHI2 || model == PSC_MODEL_PHI2CHI2 || model_is_user(model);
}

// num_potential_terms (model.h:35)
__host__ __device__ inline int model_nterms(int model) {
    if (model == PSC_MODEL_PHI2) return 1;
    if (model == PSC_MODEL_PHI2CHI2) return 2;
    return model_is_user(model) ? um_nterms(model - PSC_MODEL_USER) : 0;
}

// potential_energy(term, v) (model.h:36-75), FP64
__host__ __device__ inline double model_potential_term(int model, double gsq, int term, const double *v) {
    if (model_is_user(model)) {
        double t[PSC_MAX_TERMS] = {0, 0, 0, 0};
        um_potential<double>(model - PSC_MODEL_USER, v, t);
        return t[term];
    }
    if (model == PSC_MODEL_PHI2 || term == 0) return 0.5 * (v[0] * v[0]);
    return 0.5 * gsq * (v[0] * v[0]) * (v[1] * v[1]);
}

// dvdf(fld, v) of every field (model.h:78-85), FP64
__host__ __device__ inline void model_dvdf_all(int model, double gsq, const double *v, double *out, int nf) {
    if (model_is_user(model)) {
        um_dvdf<double>(model - PSC_MODEL_USER, v, out, nf);
        return;
    }
    if (model == PSC_MODEL_PHI2) {
        out[0] = v[0];
        return;
    }
    out[0] = v[0] + gsq * v[0] * (v[1] * v[1]);
    if (nf > 1) out[1] = gsq * (v[0] * v[0]) * v[1];
}

// effective_mass(mass_sq, v) (model.h:98-100), FP64
__host__ __device__ inline void model_effective_mass(int model, double gsq, double *m2, const double *v) {
    if (model_is_user(model)) {
        um_effective_mass<double>(model - PSC_MODEL_USER, v, m2);
        return;
    }
    if (model == PSC_MODEL_PHI2) {
        m2[0] = 1.;
        return;
    }
    m2[0] = 1. + gsq * (v[1] * v[1]);
    m2[1] = gsq * (v[0] * v[0]);
}

}  // namespace psc
