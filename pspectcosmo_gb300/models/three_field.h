// Three-field toy model in the reference's model.h interface (model.h:10-104), authored for
// this project to exercise more than two fields: the preheating inflaton phi with two
// daughter fields chi and sigma,
//
//   V = phi^2 / 2 + gsq phi^2 chi^2 / 2 + hsq phi^2 sigma^2 / 2 + lam sigma^4 / 4
//
// in program units (fStar = MPl, omegaStar = m). Terms: 0 = phi^2/2, 1 = the phi-chi
// coupling, 2 = the phi-sigma coupling plus the sigma self-interaction.
// d2Vdf2(term) follows the reference's index term = fld + fld2 (evolution.cpp:229), which
// names a pair uniquely only for up to two fields; for three fields the pairs that share
// an index (0+2 and 1+1) return the phi-sigma entry for 2, and 3, 4 are chi-sigma and
// sigma-sigma.

#include <cmath>
#include <stdexcept>
#define PHI FIELD(0)
#define CHI FIELD(1)
#define SIGMA FIELD(2)

const double gsq = 2.5e5;
const double hsq = 1.0e5;
const double lam = 1.0e3;

inline void modelinfo_(std::ofstream &info_) {
    info_ << "three-field phi^2 + g^2 phi^2 chi^2 + h^2 phi^2 sigma^2 + lambda sigma^4 Model\n";
    info_ << "V = 1/2 PHI^2 + 1/2 g^2 PHI^2 CHI^2 + 1/2 h^2 PHI^2 SIGMA^2 + 1/4 lambda SIGMA^4\n\n";
    info_ << "g^2 = " << gsq << ", h^2 = " << hsq << ", lambda = " << lam << "\n";
    info_ << "m_in_MPl = " << m_in_MPl << "\n";
    info_ << "fStar = " << fStar << "\n";
    info_ << "omegaStar = " << omegaStar << "\n";
}

inline void modelinitialize(int which_call) {
    if (which_call == 1 && nflds != 3) {
        std::cout << "Number of fields for the three-field model must be 3. Exiting." << std::endl;
        exit(1);
    }
}

const int num_potential_terms = 3;

inline double three_field_term(int term, double phi, double chi, double sigma) {
    switch (term) {
    case 0: return 0.5 * pw2(phi);
    case 1: return 0.5 * gsq * pw2(phi) * pw2(chi);
    case 2: return 0.5 * hsq * pw2(phi) * pw2(sigma) + 0.25 * lam * pw2(pw2(sigma));
    default: throw std::invalid_argument("Invalid term value in potential_energy");
    }
}

inline double potential_energy(int term, double *field_values) {
    DECLARE_INDICES
    if (field_values == NULL) {
        double sum = 0.;
        LOOP { sum += three_field_term(term, PHI, CHI, SIGMA); }
        return sum / N3;
    }
    return three_field_term(term, field_values[0], field_values[1], field_values[2]);
}

inline double dvdf(int fld, const double *field_values) {
    const double phi = field_values[0], chi = field_values[1], sigma = field_values[2];
    switch (fld) {
    case 0: return phi + gsq * phi * pw2(chi) + hsq * phi * pw2(sigma);
    case 1: return gsq * pw2(phi) * chi;
    case 2: return hsq * pw2(phi) * sigma + lam * pw2(sigma) * sigma;
    default: throw std::invalid_argument("Invalid term value in dvdf");
    }
}

inline double d2Vdf2(size_t term, double *field_values) {
    const double phi = field_values[0], chi = field_values[1], sigma = field_values[2];
    switch (term) {
    case 0: return 1. + gsq * pw2(chi) + hsq * pw2(sigma);
    case 1: return 2. * gsq * phi * chi;
    case 2: return 2. * hsq * phi * sigma;
    case 3: return 0.;
    case 4: return hsq * pw2(phi) + 3. * lam * pw2(sigma);
    default: throw std::invalid_argument("Invalid term value in d2Vdf2 ");
    }
}

inline void effective_mass(double mass_sq[], double *field_values) {
    const double phi = field_values[0], chi = field_values[1], sigma = field_values[2];
    mass_sq[0] = 1. + gsq * pw2(chi) + hsq * pw2(sigma);
    mass_sq[1] = gsq * pw2(phi);
    mass_sq[2] = hsq * pw2(phi) + 3. * lam * pw2(sigma);
}

inline void model_output(std::string ext_) {}

#undef PHI
#undef CHI
#undef SIGMA
