// CLbmSkeleton.hpp -- physical -> lattice parametrisation of the reference
// (src/CLbmSkeleton.hpp:38-199): time step from the viscosity and tau,
// lattice gravity with the step limit, lid speed = U * dt, Reynolds number.
// Every formula keeps the reference's operand order in T.
//
// Addition: initLattice() sets tau and the lid speed directly in lattice
// units (the optional <lattice> element of conf.xml), bypassing the
// reference's tau window [0.51, 2.5], which rejects the high-Reynolds
// configurations; with a subgrid model tau stays > 0.5 per cell.
#ifndef LBM_GB300_CLBMSKELETON_HPP
#define LBM_GB300_CLBMSKELETON_HPP

#include <cmath>
#include <iostream>

#include "CDomain.hpp"
#include "CError.hpp"
#include "CVector.hpp"

template <typename T>
class CLbmSkeleton {
public:
    CError error;
    bool debug = false;

    CDomain<T> domain;
    CVector<3, int> domain_cells;
    int domain_cells_count = 0;
    CVector<4, T> d_drivenCavityVelocity;

    T d_domain_x_length = 0;
    CVector<3, T> d_gravitation;
    T d_viscosity = 0;
    T mass_exchange_factor = 1;

    T d_cell_length = 0;
    T d_timestep = 0;
    T d_reynolds = 0;
    T tau = 0;
    T inv_tau = 0;
    T inv_trt_tau = 0;

    CVector<4, T> drivenCavityVelocity;
    CVector<3, T> gravitation;
    T max_sim_gravitation_length = T(0.0001);
    bool lattice_units = false;

    /** src/CLbmSkeleton.hpp:81-116 */
    void updateValues(bool info_output = false) {
        d_timestep = (d_cell_length * d_cell_length) * ((T)2.0 * tau - (T)1.0) /
                     ((T)6.0 * d_viscosity * std::sqrt(mass_exchange_factor));
        gravitation = d_gravitation * ((d_timestep * d_timestep) / d_cell_length);
        if (gravitation.length() >= max_sim_gravitation_length) {
            if (info_output) std::cout << "limiting timestep (gravitation: " << gravitation << ")" << std::endl;
            d_timestep = std::sqrt((max_sim_gravitation_length * d_cell_length) / d_gravitation.length());
            gravitation = d_gravitation * ((d_timestep * d_timestep) / d_cell_length);
            tau = (T)0.5 * (d_timestep * d_viscosity * std::sqrt(mass_exchange_factor) * (T)6.0) /
                      (d_cell_length * d_cell_length) +
                  (T)0.5;
        }
        if (tau < 0.51 || tau > 2.5) {
            error << "relaxation time " << tau << " outside the accepted window [0.51, 2.5]" << std::endl;
            error << "(runs outside it are unstable; lattice units in conf.xml bypass this check)" << std::endl;
        }
        inv_tau = (T)1.0 / tau;
        inv_trt_tau = (T)1.0 / ((T)0.5 + (T)3.0 / ((T)16.0 * tau - (T)8.0));
    }

    void setGravitation(CVector<3, T> p_d_gravitation) {
        d_gravitation = p_d_gravitation;
        updateValues();
    }

    /** src/CLbmSkeleton.hpp:132-190 */
    void init(CVector<3, T> &p_d_gravitation, T p_d_viscosity, T p_mass_exchange_factor,
              T p_max_sim_gravitation_length = 0.0001, T p_tau = (T)0.953575) {
        domain_cells = domain.getSize();
        d_domain_x_length = domain.getLength()[0];
        d_gravitation = p_d_gravitation;
        domain_cells_count = (int)domain_cells.elements();
        d_viscosity = p_d_viscosity;
        mass_exchange_factor = p_mass_exchange_factor;
        d_cell_length = d_domain_x_length / (T)domain_cells[0];
        max_sim_gravitation_length = p_max_sim_gravitation_length;
        tau = p_tau;
        updateValues(true);
        drivenCavityVelocity = d_drivenCavityVelocity * d_timestep;
        d_reynolds = d_domain_x_length * d_drivenCavityVelocity[0] / d_viscosity;
        std::cout << "dim reynolds number: " << d_reynolds << std::endl;
    }

    /** Lattice-unit parametrisation: tau and lid speed as given, gravity in
     *  lattice units, no tau window. */
    void initLattice(T p_tau, T p_lid, CVector<3, T> p_gravity = CVector<3, T>()) {
        domain_cells = domain.getSize();
        domain_cells_count = (int)domain_cells.elements();
        lattice_units = true;
        error.clear();
        if (!(p_tau > (T)0.5)) error << "lattice tau must exceed 0.5, got " << p_tau << std::endl;
        tau = p_tau;
        inv_tau = (T)1.0 / tau;
        inv_trt_tau = (T)1.0 / ((T)0.5 + (T)3.0 / ((T)16.0 * tau - (T)8.0));
        gravitation = p_gravity;
        drivenCavityVelocity = CVector<4, T>(p_lid, (T)0, (T)0, (T)1);
        d_timestep = (T)1;
        d_cell_length = (T)1;
    }

    CLbmSkeleton(CDomain<T> _domain, CVector<4, T> _drivenCavityVelocity)
        : domain(_domain), d_drivenCavityVelocity(_drivenCavityVelocity) {}
};

#endif
