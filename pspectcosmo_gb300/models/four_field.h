// Four-field toy model in the reference's model.h interface (model.h:10-104), authored for
// this project to exercise the largest field and term counts the library takes (4 and 4):
// the preheating inflaton phi with three daughter fields chi, sigma, psi,
//
//   V = phi^2 / 2 + gsq phi^2 (chi^2 + sigma^2) / 2 + hsq phi^2 psi^2 / 2
//
// in program units (fStar = MPl, omegaStar = m). Terms: 0 = phi^2/2, 1 = the phi-chi
// coupling, 2 = the phi-sigma coupling, 3 = the phi-psi coupling. d2Vdf2 follows the
// reference's index term = fld + fld2 (evolution.cpp:229), which names a pair uniquely only
// for up to two fields; it returns the diagonal entry for even indices and 0 otherwise.

#include <cmath>
#include <stdexcept>
#define PHI FIELD(0)
#define CHI FIELD(1)
#define SIGMA FIELD(2)
#define PSI FIELD(3)

const double gsq = 2.5e5;
const double hsq = 1.0e5;

inline void modelinfo_(std::ofstream &info_) {
    info_ << "four-field phi^2 + g^2 phi^2 (chi^2 + sigma^2) + h^2 phi^2 psi^2 Model\n";
    info_ << "g^2 = " << gsq << ", h^2 = " << hsq << "\n";
    info_ << "m_in_MPl = " << m_in_MPl << "\n";
    info_ << "fStar = " << fStar << "\n";
    info_ << "omegaStar = " << omegaStar << "\n";
}

inline void modelinitialize(int which_call) {
    if (which_call == 1 && nflds != 4) {
        std::cout << "Number of fields for the four-field model must be 4. Exiting." << std::endl;
        exit(1);
    }
}

const int num_potential_terms = 4;

inline double four_field_term(int term, const double *v) {
    switch (term) {
    case 0: return 0.5 * pw2(v[0]);
    case 1: return 0.5 * gsq * pw2(v[0]) * pw2(v[1]);
    case 2: return 0.5 * gsq * pw2(v[0]) * pw2(v[2]);
    case 3: return 0.5 * hsq * pw2(v[0]) * pw2(v[3]);
    default: throw std::invalid_argument("Invalid term value in potential_energy");
    }
}

inline double potential_energy(int term, double *field_values) {
    DECLARE_INDICES
    if (field_values == NULL) {
        double sum = 0.;
        LOOP {
            const double v[4] = {PHI, CHI, SIGMA, PSI};
            sum += four_field_term(term, v);
        }
        return sum / N3;
    }
    return four_field_term(term, field_values);
}

inline double dvdf(int fld, const double *field_values) {
    const double phi = field_values[0], chi = field_values[1], sigma = field_values[2], psi = field_values[3];
    switch (fld) {
    case 0: return phi + gsq * phi * (pw2(chi) + pw2(sigma)) + hsq * phi * pw2(psi);
    case 1: return gsq * pw2(phi) * chi;
    case 2: return gsq * pw2(phi) * sigma;
    case 3: return hsq * pw2(phi) * psi;
    default: throw std::invalid_argument("Invalid term value in dvdf");
    }
}

inline double d2Vdf2(size_t term, double *field_values) {
    const double phi = field_values[0], chi = field_values[1], sigma = field_values[2], psi = field_values[3];
    switch (term) {
    case 0: return 1. + gsq * (pw2(chi) + pw2(sigma)) + hsq * pw2(psi);
    case 1: return 0.;
    case 2: return gsq * pw2(phi);
    case 3: return 0.;
    case 4: return gsq * pw2(phi);
    case 5: return 0.;
    case 6: return hsq * pw2(phi);
    default: throw std::invalid_argument("Invalid term value in d2Vdf2 ");
    }
}

inline void effective_mass(double mass_sq[], double *field_values) {
    const double phi = field_values[0], chi = field_values[1], sigma = field_values[2], psi = field_values[3];
    mass_sq[0] = 1. + gsq * (pw2(chi) + pw2(sigma)) + hsq * pw2(psi);
    mass_sq[1] = gsq * pw2(phi);
    mass_sq[2] = gsq * pw2(phi);
    mass_sq[3] = hsq * pw2(phi);
}

inline void model_output(std::string ext_) {}

#undef PHI
#undef CHI
#undef SIGMA
#undef PSI
