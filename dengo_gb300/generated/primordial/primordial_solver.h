/* THIS FILE HAS BEEN AUTO-GENERATED by dengo_gb300.  DO NOT EDIT.
 *
 * C header of the GB300 solver for network "primordial".  The data struct keeps
 * the field layout of the reference's generated header
 * (rates_and_rate_tables.h.template:30-83) so host code that reads fields
 * such as Ts[] or rs_<rate>[] after a strip call keeps working; a pointer to
 * the device context is appended.
 */
#ifndef PRIMORDIAL_SOLVER_H
#define PRIMORDIAL_SOLVER_H

#define DENGO_GENERATED_HEADER 1
#include "dengo_gb300.h"

#define MAX_NCELLS DENGO_MAX_NCELLS
#define NSPECIES 10
#define DMAX(A,B) ((A) > (B) ? (A) : (B))
#define DMIN(A,B) ((A) < (B) ? (A) : (B))

#ifdef __cplusplus
extern "C" {
#endif

struct primordial_data_ {
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
    double r_k01[1024];
    double rs_k01[MAX_NCELLS];
    double drs_k01[MAX_NCELLS];
    double r_k02[1024];
    double rs_k02[MAX_NCELLS];
    double drs_k02[MAX_NCELLS];
    double r_k03[1024];
    double rs_k03[MAX_NCELLS];
    double drs_k03[MAX_NCELLS];
    double r_k04[1024];
    double rs_k04[MAX_NCELLS];
    double drs_k04[MAX_NCELLS];
    double r_k05[1024];
    double rs_k05[MAX_NCELLS];
    double drs_k05[MAX_NCELLS];
    double r_k06[1024];
    double rs_k06[MAX_NCELLS];
    double drs_k06[MAX_NCELLS];
    double r_k07[1024];
    double rs_k07[MAX_NCELLS];
    double drs_k07[MAX_NCELLS];
    double r_k08[1024];
    double rs_k08[MAX_NCELLS];
    double drs_k08[MAX_NCELLS];
    double r_k09[1024];
    double rs_k09[MAX_NCELLS];
    double drs_k09[MAX_NCELLS];
    double r_k10[1024];
    double rs_k10[MAX_NCELLS];
    double drs_k10[MAX_NCELLS];
    double r_k11[1024];
    double rs_k11[MAX_NCELLS];
    double drs_k11[MAX_NCELLS];
    double r_k12[1024];
    double rs_k12[MAX_NCELLS];
    double drs_k12[MAX_NCELLS];
    double r_k13[1024];
    double rs_k13[MAX_NCELLS];
    double drs_k13[MAX_NCELLS];
    double r_k14[1024];
    double rs_k14[MAX_NCELLS];
    double drs_k14[MAX_NCELLS];
    double r_k15[1024];
    double rs_k15[MAX_NCELLS];
    double drs_k15[MAX_NCELLS];
    double r_k16[1024];
    double rs_k16[MAX_NCELLS];
    double drs_k16[MAX_NCELLS];
    double r_k17[1024];
    double rs_k17[MAX_NCELLS];
    double drs_k17[MAX_NCELLS];
    double r_k18[1024];
    double rs_k18[MAX_NCELLS];
    double drs_k18[MAX_NCELLS];
    double r_k19[1024];
    double rs_k19[MAX_NCELLS];
    double drs_k19[MAX_NCELLS];
    double r_k21[1024];
    double rs_k21[MAX_NCELLS];
    double drs_k21[MAX_NCELLS];
    double r_k22[1024];
    double rs_k22[MAX_NCELLS];
    double drs_k22[MAX_NCELLS];
    double r_k23[1024];
    double rs_k23[MAX_NCELLS];
    double drs_k23[MAX_NCELLS];
    double c_brem_brem[1024];
    double cs_brem_brem[MAX_NCELLS];
    double dcs_brem_brem[MAX_NCELLS];
    double c_ceHI_ceHI[1024];
    double cs_ceHI_ceHI[MAX_NCELLS];
    double dcs_ceHI_ceHI[MAX_NCELLS];
    double c_ceHeI_ceHeI[1024];
    double cs_ceHeI_ceHeI[MAX_NCELLS];
    double dcs_ceHeI_ceHeI[MAX_NCELLS];
    double c_ceHeII_ceHeII[1024];
    double cs_ceHeII_ceHeII[MAX_NCELLS];
    double dcs_ceHeII_ceHeII[MAX_NCELLS];
    double c_ciHI_ciHI[1024];
    double cs_ciHI_ciHI[MAX_NCELLS];
    double dcs_ciHI_ciHI[MAX_NCELLS];
    double c_ciHeI_ciHeI[1024];
    double cs_ciHeI_ciHeI[MAX_NCELLS];
    double dcs_ciHeI_ciHeI[MAX_NCELLS];
    double c_ciHeII_ciHeII[1024];
    double cs_ciHeII_ciHeII[MAX_NCELLS];
    double dcs_ciHeII_ciHeII[MAX_NCELLS];
    double c_ciHeIS_ciHeIS[1024];
    double cs_ciHeIS_ciHeIS[MAX_NCELLS];
    double dcs_ciHeIS_ciHeIS[MAX_NCELLS];
    double c_gammah_gammah[1024];
    double cs_gammah_gammah[MAX_NCELLS];
    double dcs_gammah_gammah[MAX_NCELLS];
    double c_gloverabel08_gaH2[1024];
    double cs_gloverabel08_gaH2[MAX_NCELLS];
    double dcs_gloverabel08_gaH2[MAX_NCELLS];
    double c_gloverabel08_gaHI[1024];
    double cs_gloverabel08_gaHI[MAX_NCELLS];
    double dcs_gloverabel08_gaHI[MAX_NCELLS];
    double c_gloverabel08_gaHe[1024];
    double cs_gloverabel08_gaHe[MAX_NCELLS];
    double dcs_gloverabel08_gaHe[MAX_NCELLS];
    double c_gloverabel08_gaHp[1024];
    double cs_gloverabel08_gaHp[MAX_NCELLS];
    double dcs_gloverabel08_gaHp[MAX_NCELLS];
    double c_gloverabel08_gael[1024];
    double cs_gloverabel08_gael[MAX_NCELLS];
    double dcs_gloverabel08_gael[MAX_NCELLS];
    double c_gloverabel08_gphdl[1024];
    double cs_gloverabel08_gphdl[MAX_NCELLS];
    double dcs_gloverabel08_gphdl[MAX_NCELLS];
    double c_gloverabel08_gpldl[1024];
    double cs_gloverabel08_gpldl[MAX_NCELLS];
    double dcs_gloverabel08_gpldl[MAX_NCELLS];
    double c_h2formation_h2mcool[1024];
    double cs_h2formation_h2mcool[MAX_NCELLS];
    double dcs_h2formation_h2mcool[MAX_NCELLS];
    double c_h2formation_h2mheat[1024];
    double cs_h2formation_h2mheat[MAX_NCELLS];
    double dcs_h2formation_h2mheat[MAX_NCELLS];
    double c_reHII_reHII[1024];
    double cs_reHII_reHII[MAX_NCELLS];
    double dcs_reHII_reHII[MAX_NCELLS];
    double c_reHeII1_reHeII1[1024];
    double cs_reHeII1_reHeII1[MAX_NCELLS];
    double dcs_reHeII1_reHeII1[MAX_NCELLS];
    double c_reHeII2_reHeII2[1024];
    double cs_reHeII2_reHeII2[MAX_NCELLS];
    double dcs_reHeII2_reHeII2[MAX_NCELLS];
    double c_reHeIII_reHeIII[1024];
    double cs_reHeIII_reHeIII[MAX_NCELLS];
    double dcs_reHeIII_reHeIII[MAX_NCELLS];
    int bin_id[MAX_NCELLS];
    int ncells;
    void *gpu;
};

DENGO_DECLARE_NETWORK(primordial)
DENGO_DECLARE_NETWORK_NOALLOC(primordial)

#ifdef __cplusplus
}
/* The reference's C++ prototype takes dt by reference
 * (rates_and_rate_tables.h.template:88-91). */
inline double dengo_evolve_primordial(double dtf, double &dt, double z, double *input,
                                   double *rtol, double *atol, long long dims,
                                   primordial_data *data)
{
    return dengo_evolve_primordial(dtf, &dt, z, input, rtol, atol, dims, data);
}
#endif
#endif
