// Two-field preheating model V = m^2 phi^2 / 2 + g^2 phi^2 chi^2 / 2, written
// in the reference's model.h interface (model.h:10-104: modelinfo_,
// modelinitialize, num_potential_terms, potential_energy, dvdf, d2Vdf2,
// effective_mass, model_output) so the reference's own sources can be built
// with it as the oracle for the two-field configurations. The reference ships
// only the single-field phi^2 model; this file is authored for this project.
//
// Program units (fStar = MPl, omegaStar = m): V = phi^2/2 + gsq phi^2 chi^2/2
// with gsq = g^2 MPl^2 / m^2 (2.5e5 for the preheating benchmark).
// d2Vdf2(term) indexes term = fld + fld2 as evolution.cpp:229 does:
// 0 = phi-phi, 1 = phi-chi, 2 = chi-chi.

#include <cmath>
#include <stdexcept>
#define PHI FIELD(0)
#define CHI FIELD(1)

#ifndef PSC_MODEL_GSQ
#define PSC_MODEL_GSQ 2.5e5
#endif
const double gsq = PSC_MODEL_GSQ;

inline void modelinfo_(std::ofstream &info_) {
    info_ << "two-field phi^2 + g^2 phi^2 chi^2 Model\n";
    info_ << "V = 1/2 m^2 PHI^2 + 1/2 g^2 PHI^2 CHI^2\n\n";
    info_ << "m_in_MPl = " << m_in_MPl << "\n";
    info_ << "g^2 (program units) = " << gsq << "\n";
    info_ << "fStar = " << fStar << "\n";
    info_ << "omegaStar = " << omegaStar << "\n";
}

inline void modelinitialize(int which_call) {
    if (which_call == 1 && nflds != 2) {
        std::cout << "Number of fields for the phi^2 chi^2 model must be 2. Exiting." << std::endl;
        exit(1);
    }
}

const int num_potential_terms = 2;

inline double potential_term_at(int term, double phi, double chi) {
    switch (term) {
    case 0: return 0.5 * pw2(phi);
    case 1: return 0.5 * gsq * pw2(phi) * pw2(chi);
    default: throw std::invalid_argument("Invalid term value in potential_energy");
    }
}

inline double potential_energy(int term, double *field_values) {
    DECLARE_INDICES
    if (field_values == NULL) {
        double sum = 0.;
        LOOP { sum += potential_term_at(term, PHI, CHI); }
        return sum / N3;
    }
    return potential_term_at(term, field_values[0], field_values[1]);
}

inline double dvdf(int fld, const double *field_values) {
    const double phi = field_values[0], chi = field_values[1];
    switch (fld) {
    case 0: return phi + gsq * phi * pw2(chi);
    case 1: return gsq * pw2(phi) * chi;
    default: throw std::invalid_argument("Invalid term value in dvdf");
    }
}

inline double d2Vdf2(size_t term, double *field_values) {
    const double phi = field_values[0], chi = field_values[1];
    switch (term) {
    case 0: return 1. + gsq * pw2(chi);
    case 1: return 2. * gsq * phi * chi;
    case 2: return gsq * pw2(phi);
    default: throw std::invalid_argument("Invalid term value in d2Vdf2 ");
    }
}

inline void effective_mass(double mass_sq[], double *field_values) {
    mass_sq[0] = 1. + gsq * pw2(field_values[1]);
    mass_sq[1] = gsq * pw2(field_values[0]);
}

inline void model_output(std::string ext_) {}

#undef PHI
#undef CHI
