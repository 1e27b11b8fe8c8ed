/* THIS FILE HAS BEEN AUTO-GENERATED by dengo_gb300.  DO NOT EDIT.
 *
 * C header of the GB300 solver for network "oxygen".  The data struct keeps
 * the field layout of the reference's generated header
 * (rates_and_rate_tables.h.template:30-83) so host code that reads fields
 * such as Ts[] or rs_<rate>[] after a strip call keeps working; a pointer to
 * the device context is appended.
 */
#ifndef OXYGEN_SOLVER_H
#define OXYGEN_SOLVER_H

#define DENGO_GENERATED_HEADER 1
#include "dengo_gb300.h"

#define MAX_NCELLS DENGO_MAX_NCELLS
#define NSPECIES 16
#define DMAX(A,B) ((A) > (B) ? (A) : (B))
#define DMIN(A,B) ((A) < (B) ? (A) : (B))

#ifdef __cplusplus
extern "C" {
#endif

struct oxygen_data_ {
    double dbin;
    double idbin;
    double bounds[2];
    int nbins;
    double d_zbin;
    double id_zbin;
    double z_bounds[2];
    int n_zbins;
    double current_z;
    double zdef;
    double dz;
    double Ts[MAX_NCELLS];
    double Tdef[MAX_NCELLS];
    double dT[MAX_NCELLS];
    double logTs[MAX_NCELLS];
    double invTs[MAX_NCELLS];
    double dTs_ge[MAX_NCELLS];
    double r_H_1_i[8192];
    double rs_H_1_i[MAX_NCELLS];
    double drs_H_1_i[MAX_NCELLS];
    double r_H_2_r[8192];
    double rs_H_2_r[MAX_NCELLS];
    double drs_H_2_r[MAX_NCELLS];
    double r_He_1_i[8192];
    double rs_He_1_i[MAX_NCELLS];
    double drs_He_1_i[MAX_NCELLS];
    double r_He_2_i[8192];
    double rs_He_2_i[MAX_NCELLS];
    double drs_He_2_i[MAX_NCELLS];
    double r_He_2_r[8192];
    double rs_He_2_r[MAX_NCELLS];
    double drs_He_2_r[MAX_NCELLS];
    double r_He_3_r[8192];
    double rs_He_3_r[MAX_NCELLS];
    double drs_He_3_r[MAX_NCELLS];
    double r_O_1_i[8192];
    double rs_O_1_i[MAX_NCELLS];
    double drs_O_1_i[MAX_NCELLS];
    double r_O_2_i[8192];
    double rs_O_2_i[MAX_NCELLS];
    double drs_O_2_i[MAX_NCELLS];
    double r_O_2_r[8192];
    double rs_O_2_r[MAX_NCELLS];
    double drs_O_2_r[MAX_NCELLS];
    double r_O_3_i[8192];
    double rs_O_3_i[MAX_NCELLS];
    double drs_O_3_i[MAX_NCELLS];
    double r_O_3_r[8192];
    double rs_O_3_r[MAX_NCELLS];
    double drs_O_3_r[MAX_NCELLS];
    double r_O_4_i[8192];
    double rs_O_4_i[MAX_NCELLS];
    double drs_O_4_i[MAX_NCELLS];
    double r_O_4_r[8192];
    double rs_O_4_r[MAX_NCELLS];
    double drs_O_4_r[MAX_NCELLS];
    double r_O_5_i[8192];
    double rs_O_5_i[MAX_NCELLS];
    double drs_O_5_i[MAX_NCELLS];
    double r_O_5_r[8192];
    double rs_O_5_r[MAX_NCELLS];
    double drs_O_5_r[MAX_NCELLS];
    double r_O_6_i[8192];
    double rs_O_6_i[MAX_NCELLS];
    double drs_O_6_i[MAX_NCELLS];
    double r_O_6_r[8192];
    double rs_O_6_r[MAX_NCELLS];
    double drs_O_6_r[MAX_NCELLS];
    double r_O_7_i[8192];
    double rs_O_7_i[MAX_NCELLS];
    double drs_O_7_i[MAX_NCELLS];
    double r_O_7_r[8192];
    double rs_O_7_r[MAX_NCELLS];
    double drs_O_7_r[MAX_NCELLS];
    double r_O_8_i[8192];
    double rs_O_8_i[MAX_NCELLS];
    double drs_O_8_i[MAX_NCELLS];
    double r_O_8_r[8192];
    double rs_O_8_r[MAX_NCELLS];
    double drs_O_8_r[MAX_NCELLS];
    double r_O_9_r[8192];
    double rs_O_9_r[MAX_NCELLS];
    double drs_O_9_r[MAX_NCELLS];
    double c_H_1_c_H_1_c[8192];
    double cs_H_1_c_H_1_c[MAX_NCELLS];
    double dcs_H_1_c_H_1_c[MAX_NCELLS];
    double c_H_2_c_H_2_c[8192];
    double cs_H_2_c_H_2_c[MAX_NCELLS];
    double dcs_H_2_c_H_2_c[MAX_NCELLS];
    double c_He_1_c_He_1_c[8192];
    double cs_He_1_c_He_1_c[MAX_NCELLS];
    double dcs_He_1_c_He_1_c[MAX_NCELLS];
    double c_He_2_c_He_2_c[8192];
    double cs_He_2_c_He_2_c[MAX_NCELLS];
    double dcs_He_2_c_He_2_c[MAX_NCELLS];
    double c_He_3_c_He_3_c[8192];
    double cs_He_3_c_He_3_c[MAX_NCELLS];
    double dcs_He_3_c_He_3_c[MAX_NCELLS];
    double c_O_1_c_O_1_c[8192];
    double cs_O_1_c_O_1_c[MAX_NCELLS];
    double dcs_O_1_c_O_1_c[MAX_NCELLS];
    double c_O_2_c_O_2_c[8192];
    double cs_O_2_c_O_2_c[MAX_NCELLS];
    double dcs_O_2_c_O_2_c[MAX_NCELLS];
    double c_O_3_c_O_3_c[8192];
    double cs_O_3_c_O_3_c[MAX_NCELLS];
    double dcs_O_3_c_O_3_c[MAX_NCELLS];
    double c_O_4_c_O_4_c[8192];
    double cs_O_4_c_O_4_c[MAX_NCELLS];
    double dcs_O_4_c_O_4_c[MAX_NCELLS];
    double c_O_5_c_O_5_c[8192];
    double cs_O_5_c_O_5_c[MAX_NCELLS];
    double dcs_O_5_c_O_5_c[MAX_NCELLS];
    double c_O_6_c_O_6_c[8192];
    double cs_O_6_c_O_6_c[MAX_NCELLS];
    double dcs_O_6_c_O_6_c[MAX_NCELLS];
    double c_O_7_c_O_7_c[8192];
    double cs_O_7_c_O_7_c[MAX_NCELLS];
    double dcs_O_7_c_O_7_c[MAX_NCELLS];
    double c_O_8_c_O_8_c[8192];
    double cs_O_8_c_O_8_c[MAX_NCELLS];
    double dcs_O_8_c_O_8_c[MAX_NCELLS];
    double c_O_9_c_O_9_c[8192];
    double cs_O_9_c_O_9_c[MAX_NCELLS];
    double dcs_O_9_c_O_9_c[MAX_NCELLS];
    int bin_id[MAX_NCELLS];
    int ncells;
    void *gpu;
};

DENGO_DECLARE_NETWORK(oxygen)
DENGO_DECLARE_NETWORK_NOALLOC(oxygen)

#ifdef __cplusplus
}
/* The reference's C++ prototype takes dt by reference
 * (rates_and_rate_tables.h.template:88-91). */
inline double dengo_evolve_oxygen(double dtf, double &dt, double z, double *input,
                                   double *rtol, double *atol, long long dims,
                                   oxygen_data *data)
{
    return dengo_evolve_oxygen(dtf, &dt, z, input, rtol, atol, dims, data);
}
#endif
#endif
