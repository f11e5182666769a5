// Single-field chaotic inflation V = m^2 phi^2 / 2 in program units (V = phi^2 / 2 with
// omegaStar = m), written in the reference's model.h interface (model.h:10-104:
// modelinfo_, modelinitialize, num_potential_terms, potential_energy, dvdf, d2Vdf2,
// effective_mass, model_output). It is the physics of the model the reference ships,
// kept here so that the user-model path of this library has a one-field model that every
// build compiles; the library's built-in PSC_MODEL_PHI2 is the same potential.

#include <cmath>
#include <stdexcept>
#define PHI FIELD(0)

inline void modelinfo_(std::ofstream &info_) {
    info_ << "single phi^2 Model\n";
    info_ << "V = 1/2 * m_in_MPl^2 * PHI^2 \n\n";
    info_ << "m_in_MPl = " << m_in_MPl << "\n";
    info_ << "fStar = " << fStar << "\n";
    info_ << "omegaStar = " << omegaStar << "\n";
}

inline void modelinitialize(int which_call) {
    if (which_call == 1 && nflds != 1) {
        std::cout << "Number of fields for the phi^2 model must be 1. Exiting." << std::endl;
        exit(1);
    }
}

const int num_potential_terms = 1;

inline double potential_energy(int term, double *field_values) {
    DECLARE_INDICES
    double sum = 0.;
    if (field_values == NULL) {
        LOOP { sum += pw2(PHI); }
        sum /= N3;
    } else {
        sum = pw2(field_values[0]);
    }
    if (term != 0) throw std::invalid_argument("Invalid term value in potential_energy");
    return 0.5 * sum;
}

inline double dvdf(int fld, const double *field_values) {
    if (fld != 0) throw std::invalid_argument("Invalid term value in dvdf");
    return field_values[0];
}

inline double d2Vdf2(size_t term, double *field_values) {
    if (term != 0) throw std::invalid_argument("Invalid term value in d2Vdf2 ");
    return 1.;
}

inline void effective_mass(double mass_sq[], double *field_values) { mass_sq[0] = 1.; }

inline void model_output(std::string ext_) {}

#undef PHI
