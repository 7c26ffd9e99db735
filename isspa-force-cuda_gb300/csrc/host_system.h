// host_system.h -- host-side system state assembled from the reference's
// input files (prmtop, isspatop, rst7, US config) or from caller arrays.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "isspa_gb300.h"

struct isspa_host_system {
    int n_atoms = 0;
    std::vector<float> pos;       // [n][4] x y z q/sqrt(eps)
    std::vector<float> vel;       // [n][4] vx vy vz mass(H->12)
    std::vector<float> raw_mass;  // [n]
    int n_lj_types = 0;
    std::vector<int> lj_type, nb_parm_index;
    std::vector<float> lj_ab;     // [ntt][2]
    std::vector<int> n_excl_cum, excl_list;
    std::vector<int> bond_atoms;  // [nb][3]
    std::vector<float> bond_params;
    int n_bond_types = 0;
    std::vector<int> angle_atoms;  // [na][4]
    std::vector<float> angle_params;
    int n_angle_types = 0;
    std::vector<int> dih_atoms, dih_types;  // [nd][4], [nd]
    std::vector<float> dih_params, scaled14;
    int n_dih_types = 0;
    // IS-SPA
    bool have_isspa = false;
    std::vector<int> isspa_type;
    int n_isspa_types = 0;
    std::vector<float> rmax;
    int n_g = 0, n_e = 0, n_f = 0;
    std::vector<float> g_table, e_table, f_table;
    float g_r0 = 0, g_dr = 1, e_r0 = 0, e_dr = 1, f_r0 = 0, f_dr = 1;
    // umbrella
    int us_on = 0;
    std::vector<int> bias_list;  // [nb][2]
    float us_k = 0, us_x0 = 0;
    // run
    int n_mc = 0;
    float box = 0, kT = 0, dt = 0, pnu = 0;
    uint64_t seed = 0;
};

namespace isspa {
// Fill a host system from a caller's description (deep copy).
int host_system_from_desc(const isspa_system_desc &d, isspa_host_system &s);
// Seeded Maxwell-Boltzmann velocities (replaces atom::initialize_velocities).
void init_velocities(isspa_host_system &s, uint64_t seed);
}  // namespace isspa
