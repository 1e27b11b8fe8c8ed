/*
 * ORACLE -- test infrastructure, not part of the product.
 * Generated by oracle/gen_oracle.py for network "primordial_compton"; do not edit.
 *
 * Per-network pieces of the reference's generated solver, restated with the
 * reference's expression text (sympy ccode) and statement order:
 *   setup/bins          rates_and_rate_tables.C.template:17-37
 *   calculate_temperature  rates_and_rate_tables.C.template:309-350
 *   interpolate_rates   rates_and_rate_tables.C.template:362-455
 *   calculate_rhs       rates_and_rate_tables.C.template:460-522
 *   calculate_jacobian  rates_and_rate_tables.C.template:527-599
 *   ensure_electron_consistency  rates_and_rate_tables.C.template:604-630
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../be_oracle.h"

/* log T of calculate_temperature: the reference's libm log, or (built with
 * -DDGO_LOG=dgo_crlog) a correctly rounded one, for telling libm rounding
 * apart from other differences */
#ifndef DGO_LOG
#define DGO_LOG log
#endif

#define MAX_NCELLS 1024
#define NCHEM 10
#define NTAB 45
#define NT_LEN 1024
#define NZ_LEN 0
#define TLEN (NT_LEN > NZ_LEN ? NT_LEN : NZ_LEN)

typedef struct {
    double dbin, idbin, bounds[2];
    int nbins;
    double d_zbin, id_zbin, z_bounds[2];
    int n_zbins;
    double current_z, zdef, dz;
    double Ts[MAX_NCELLS], Tdef[MAX_NCELLS], dT[MAX_NCELLS], logTs[MAX_NCELLS];
    double invTs[MAX_NCELLS], dTs_ge[MAX_NCELLS];
    double r[NTAB][TLEN];
    double rs[NTAB][MAX_NCELLS];
    double drs[NTAB][MAX_NCELLS];
    int bin_id[MAX_NCELLS];
    int ncells;
} dgo_primordial_compton_data;

static const int zdep[NTAB > 0 ? NTAB : 1] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,  };

static void *alloc_data(const double *const *tables)
{
    int k;
    dgo_primordial_compton_data *data = (dgo_primordial_compton_data *)calloc(1, sizeof(*data));
    data->bounds[0] = 1.0;
    data->bounds[1] = 1000000000.0;
    data->nbins = NT_LEN - 1;
    data->dbin = (log(data->bounds[1]) - log(data->bounds[0])) / data->nbins;
    data->idbin = 1.0L / data->dbin;
    data->z_bounds[0] = 0.0;
    data->z_bounds[1] = 0.0;
    data->n_zbins = NZ_LEN - 1;
    data->d_zbin = (log(data->z_bounds[1] + 1.0) - log(data->z_bounds[0] + 1.0)) / data->n_zbins;
    data->id_zbin = 1.0L / data->d_zbin;
    for (k = 0; k < NTAB; k++)
        memcpy(data->r[k], tables[k], sizeof(double) * (zdep[k] ? NZ_LEN : NT_LEN));
    return data;
}

static void free_data(void *d) { free(d); }
static void set_z(void *d, double z) { ((dgo_primordial_compton_data *)d)->current_z = z; }
static const double *get_Ts(const void *d) { return ((const dgo_primordial_compton_data *)d)->Ts; }

void dgo_primordial_compton_calculate_temperature(dgo_primordial_compton_data *data, double *input,
                                            int nstrip, int nchem)
{
    int i, j;
    double density;
    double kb = 1.3806504e-16;
    double mh = 1.67e-24;
    double gamma = 5.e0/3.e0;
    double gammaH2 = 7.e0/5.e0;
    (void)gammaH2;
    double H2_1;
    double H2_2;
    double H_1;
    double H_2;
    double H_m0;
    double He_1;
    double He_2;
    double He_3;
    double de;
    double ge;
    for (i = 0; i < nstrip; i++) {
        j = i * nchem;
        H2_1 = input[j];
        j++;
        H2_2 = input[j];
        j++;
        H_1 = input[j];
        j++;
        H_2 = input[j];
        j++;
        H_m0 = input[j];
        j++;
        He_1 = input[j];
        j++;
        He_2 = input[j];
        j++;
        He_3 = input[j];
        j++;
        de = input[j];
        j++;
        ge = input[j];
        j++;
        density = 2.0*H2_1 + 2.0*H2_2 + 1.0079400000000001*H_1 + 1.0079400000000001*H_2 + 1.0079400000000001*H_m0 + 4.0026020000000004*He_1 + 4.0026020000000004*He_2 + 4.0026020000000004*He_3;
        data->Ts[i] = density*ge*mh/(kb*(H2_1/(gamma - 1.0) + H2_2/(gamma - 1.0) + H_1/(gamma - 1.0) + H_2/(gamma - 1.0) + H_m0/(gamma - 1.0) + He_1/(gamma - 1.0) + He_2/(gamma - 1.0) + He_3/(gamma - 1.0) + de/(gamma - 1.0)));
        if (data->Ts[i] < data->bounds[0]) {
            data->Ts[i] = data->bounds[0];
        } else if (data->Ts[i] > data->bounds[1]) {
            data->Ts[i] = data->bounds[1];
        }
        data->logTs[i] = DGO_LOG(data->Ts[i]);
        data->invTs[i] = 1.0 / data->Ts[i];
        data->dTs_ge[i] = density*mh/(kb*(H2_1/(gamma - 1.0) + H2_2/(gamma - 1.0) + H_1/(gamma - 1.0) + H_2/(gamma - 1.0) + H_m0/(gamma - 1.0) + He_1/(gamma - 1.0) + He_2/(gamma - 1.0) + He_3/(gamma - 1.0) + de/(gamma - 1.0)));
    }
}

void dgo_primordial_compton_interpolate_rates(dgo_primordial_compton_data *data, int nstrip)
{
    int i, k, bin_id, zbin_id = 0;
    double lb, t1, t2, lbz, z1, z2;
    int no_photo = 0;
    lb = log(data->bounds[0]);
    lbz = log(data->z_bounds[0] + 1.0);
    for (i = 0; i < nstrip; i++) {
        data->bin_id[i] = bin_id = (int)(data->idbin * (data->logTs[i] - lb));
        if (data->bin_id[i] <= 0) {
            data->bin_id[i] = 0;
        } else if (data->bin_id[i] >= data->nbins) {
            data->bin_id[i] = data->nbins - 1;
        }
        t1 = (lb + (bin_id) * data->dbin);
        t2 = (lb + (bin_id + 1) * data->dbin);
        data->Tdef[i] = (data->logTs[i] - t1) / (t2 - t1);
        data->dT[i] = (t2 - t1);
    }
    if ((data->current_z >= data->z_bounds[0]) && (data->current_z < data->z_bounds[1])) {
        zbin_id = (int)(data->id_zbin * (log(data->current_z + 1.0) - lbz));
        if (zbin_id <= 0) {
            zbin_id = 0;
        } else if (zbin_id >= data->n_zbins) {
            zbin_id = data->n_zbins - 1;
        }
        z1 = (lbz + (zbin_id) * data->d_zbin);
        z2 = (lbz + (zbin_id + 1) * data->d_zbin);
        data->zdef = (log(data->current_z + 1.0) - z1) / (z2 - z1);
        data->dz = (exp(z2) - exp(z1));
    } else {
        no_photo = 1;
    }
    for (k = 0; k < NTAB; k++) {
        const double *r = data->r[k];
        if (!zdep[k]) {
            for (i = 0; i < nstrip; i++) {
                bin_id = data->bin_id[i];
                data->rs[k][i] = r[bin_id] + data->Tdef[i] * (r[bin_id + 1] - r[bin_id]);
                data->drs[k][i] = (r[bin_id + 1] - r[bin_id]);
                data->drs[k][i] /= data->dT[i];
                data->drs[k][i] *= data->invTs[i];
            }
        } else {
            for (i = 0; i < nstrip; i++) {
                if (no_photo) {
                    data->rs[k][i] = 0.0;
                    data->drs[k][i] = 0.0;
                } else {
                    data->rs[k][i] = r[zbin_id] + data->zdef * (r[zbin_id + 1] - r[zbin_id]);
                    data->drs[k][i] = (r[zbin_id + 1] - r[zbin_id]);
                    data->drs[k][i] /= data->dz;
                }
            }
        }
    }
}

int dgo_calculate_rhs_primordial_compton(double *input, double *rhs, int nstrip, int nchem,
                                   void *sdata)
{
    dgo_primordial_compton_data *data = (dgo_primordial_compton_data *)sdata;
    int i, j;
    dgo_primordial_compton_calculate_temperature(data, input, nstrip, nchem);
    dgo_primordial_compton_interpolate_rates(data, nstrip);
    double *k01 = data->rs[0];
    double *k02 = data->rs[1];
    double *k03 = data->rs[2];
    double *k04 = data->rs[3];
    double *k05 = data->rs[4];
    double *k06 = data->rs[5];
    double *k07 = data->rs[6];
    double *k08 = data->rs[7];
    double *k09 = data->rs[8];
    double *k10 = data->rs[9];
    double *k11 = data->rs[10];
    double *k12 = data->rs[11];
    double *k13 = data->rs[12];
    double *k14 = data->rs[13];
    double *k15 = data->rs[14];
    double *k16 = data->rs[15];
    double *k17 = data->rs[16];
    double *k18 = data->rs[17];
    double *k19 = data->rs[18];
    double *k21 = data->rs[19];
    double *k22 = data->rs[20];
    double *k23 = data->rs[21];
    double *brem_brem = data->rs[22];
    double *ceHI_ceHI = data->rs[23];
    double *ceHeI_ceHeI = data->rs[24];
    double *ceHeII_ceHeII = data->rs[25];
    double *ciHI_ciHI = data->rs[26];
    double *ciHeI_ciHeI = data->rs[27];
    double *ciHeII_ciHeII = data->rs[28];
    double *ciHeIS_ciHeIS = data->rs[29];
    double *compton_comp = data->rs[30];
    double *gammah_gammah = data->rs[31];
    double *gloverabel08_gaH2 = data->rs[32];
    double *gloverabel08_gaHI = data->rs[33];
    double *gloverabel08_gaHe = data->rs[34];
    double *gloverabel08_gaHp = data->rs[35];
    double *gloverabel08_gael = data->rs[36];
    double *gloverabel08_gphdl = data->rs[37];
    double *gloverabel08_gpldl = data->rs[38];
    double *h2formation_h2mcool = data->rs[39];
    double *h2formation_h2mheat = data->rs[40];
    double *reHII_reHII = data->rs[41];
    double *reHeII1_reHeII1 = data->rs[42];
    double *reHeII2_reHeII2 = data->rs[43];
    double *reHeIII_reHeIII = data->rs[44];
    double H2_1;
    double H2_2;
    double H_1;
    double H_2;
    double H_m0;
    double He_1;
    double He_2;
    double He_3;
    double de;
    double ge;
    double z;
    double T;
    double mh = 1.67e-24;
    double mdensity;
    for (i = 0; i < nstrip; i++) {
        j = i * nchem;
        mdensity = 0.0;
        T = data->Ts[i];
        z = data->current_z;
        (void)T; (void)z;
        H2_1 = input[j];
        mdensity += H2_1;
        if (H2_1 < 0.0) return 1;
        j++;
        H2_2 = input[j];
        mdensity += H2_2;
        if (H2_2 < 0.0) return 1;
        j++;
        H_1 = input[j];
        mdensity += H_1;
        if (H_1 < 0.0) return 1;
        j++;
        H_2 = input[j];
        mdensity += H_2;
        if (H_2 < 0.0) return 1;
        j++;
        H_m0 = input[j];
        mdensity += H_m0;
        if (H_m0 < 0.0) return 1;
        j++;
        He_1 = input[j];
        mdensity += He_1;
        if (He_1 < 0.0) return 1;
        j++;
        He_2 = input[j];
        mdensity += He_2;
        if (He_2 < 0.0) return 1;
        j++;
        He_3 = input[j];
        mdensity += He_3;
        if (He_3 < 0.0) return 1;
        j++;
        de = input[j];
        if (de < 0.0) return 1;
        j++;
        ge = input[j];
        if (ge < 0.0) return 1;
        j++;
        mdensity *= mh;
        j = i * nchem;
        rhs[j] = k08[i]*H_1*H_m0 + k10[i]*H2_2*H_1 - k11[i]*H2_1*H_2 - k12[i]*H2_1*de - k13[i]*H2_1*H_1 + k19[i]*H2_2*H_m0 + k21[i]*H2_1*pow(H_1, 2) + k22[i]*pow(H_1, 3) - k23[i]*pow(H2_1, 2);
        j++;
        rhs[j] = k09[i]*H_1*H_2 - k10[i]*H2_2*H_1 + k11[i]*H2_1*H_2 + k17[i]*H_2*H_m0 - k18[i]*H2_2*de - k19[i]*H2_2*H_m0;
        j++;
        rhs[j] = -k01[i]*H_1*de + k02[i]*H_2*de - k07[i]*H_1*de - k08[i]*H_1*H_m0 - k09[i]*H_1*H_2 - k10[i]*H2_2*H_1 + k11[i]*H2_1*H_2 + 2*k13[i]*H2_1*H_1 + k14[i]*H_m0*de + k15[i]*H_1*H_m0 + 2*k16[i]*H_2*H_m0 + 2*k18[i]*H2_2*de + k19[i]*H2_2*H_m0 - 2*k21[i]*H2_1*pow(H_1, 2) - 2*k22[i]*pow(H_1, 3) + 2*k23[i]*pow(H2_1, 2);
        j++;
        rhs[j] = k01[i]*H_1*de - k02[i]*H_2*de - k09[i]*H_1*H_2 + k10[i]*H2_2*H_1 - k11[i]*H2_1*H_2 + 2*k12[i]*H2_1*de - k16[i]*H_2*H_m0 - k17[i]*H_2*H_m0;
        j++;
        rhs[j] = k07[i]*H_1*de - k08[i]*H_1*H_m0 - k14[i]*H_m0*de - k15[i]*H_1*H_m0 - k16[i]*H_2*H_m0 - k17[i]*H_2*H_m0 - k19[i]*H2_2*H_m0;
        j++;
        rhs[j] = -k03[i]*He_1*de + k04[i]*He_2*de;
        j++;
        rhs[j] = k03[i]*He_1*de - k04[i]*He_2*de - k05[i]*He_2*de + k06[i]*He_3*de;
        j++;
        rhs[j] = k05[i]*He_2*de - k06[i]*He_3*de;
        j++;
        rhs[j] = k01[i]*H_1*de - k02[i]*H_2*de + k03[i]*He_1*de - k04[i]*He_2*de + k05[i]*He_2*de - k06[i]*He_3*de - k07[i]*H_1*de + k08[i]*H_1*H_m0 + k14[i]*H_m0*de + k15[i]*H_1*H_m0 + k17[i]*H_2*H_m0 - k18[i]*H2_2*de;
        j++;
        rhs[j] = -H2_1*H_1*h2formation_h2mcool[i] - H2_1*gloverabel08_gphdl[i]/(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0) + pow(H_1, 3)*h2formation_h2mheat[i] - H_1*ceHI_ceHI[i]*de - H_1*ciHI_ciHI[i]*de - H_2*de*reHII_reHII[i] - He_1*ciHeI_ciHeI[i]*de - He_2*ceHeII_ceHeII[i]*de - He_2*ceHeI_ceHeI[i]*pow(de, 2) - He_2*ciHeII_ciHeII[i]*de - He_2*ciHeIS_ciHeIS[i]*pow(de, 2) - He_2*de*reHeII1_reHeII1[i] - He_2*de*reHeII2_reHeII2[i] - He_3*de*reHeIII_reHeIII[i] - brem_brem[i]*de*(H_2 + He_2 + 4.0*He_3) - compton_comp[i]*de*pow(z + 1.0, 4)*(T - 2.73*z - 2.73);
        rhs[j] /= mdensity;
        j++;
    }
    return 0;
}

int dgo_calculate_jacobian_primordial_compton(double *input, double *Joutput, int nstrip,
                                        int nchem, void *sdata)
{
    dgo_primordial_compton_data *data = (dgo_primordial_compton_data *)sdata;
    int i, j;
    double *Tge = data->dTs_ge;
    double *k01 = data->rs[0];
    double *k02 = data->rs[1];
    double *k03 = data->rs[2];
    double *k04 = data->rs[3];
    double *k05 = data->rs[4];
    double *k06 = data->rs[5];
    double *k07 = data->rs[6];
    double *k08 = data->rs[7];
    double *k09 = data->rs[8];
    double *k10 = data->rs[9];
    double *k11 = data->rs[10];
    double *k12 = data->rs[11];
    double *k13 = data->rs[12];
    double *k14 = data->rs[13];
    double *k15 = data->rs[14];
    double *k16 = data->rs[15];
    double *k17 = data->rs[16];
    double *k18 = data->rs[17];
    double *k19 = data->rs[18];
    double *k21 = data->rs[19];
    double *k22 = data->rs[20];
    double *k23 = data->rs[21];
    double *brem_brem = data->rs[22];
    double *ceHI_ceHI = data->rs[23];
    double *ceHeI_ceHeI = data->rs[24];
    double *ceHeII_ceHeII = data->rs[25];
    double *ciHI_ciHI = data->rs[26];
    double *ciHeI_ciHeI = data->rs[27];
    double *ciHeII_ciHeII = data->rs[28];
    double *ciHeIS_ciHeIS = data->rs[29];
    double *compton_comp = data->rs[30];
    double *gammah_gammah = data->rs[31];
    double *gloverabel08_gaH2 = data->rs[32];
    double *gloverabel08_gaHI = data->rs[33];
    double *gloverabel08_gaHe = data->rs[34];
    double *gloverabel08_gaHp = data->rs[35];
    double *gloverabel08_gael = data->rs[36];
    double *gloverabel08_gphdl = data->rs[37];
    double *gloverabel08_gpldl = data->rs[38];
    double *h2formation_h2mcool = data->rs[39];
    double *h2formation_h2mheat = data->rs[40];
    double *reHII_reHII = data->rs[41];
    double *reHeII1_reHeII1 = data->rs[42];
    double *reHeII2_reHeII2 = data->rs[43];
    double *reHeIII_reHeIII = data->rs[44];
    double H2_1;
    double H2_2;
    double H_1;
    double H_2;
    double H_m0;
    double He_1;
    double He_2;
    double He_3;
    double de;
    double ge;
    double z;
    double T;
    double mh = 1.67e-24;
    double mdensity;
    for (i = 0; i < nstrip; i++) {
        j = i * nchem;
        mdensity = 0.0;
        T = data->Ts[i];
        z = data->current_z;
        (void)T; (void)z;
        H2_1 = input[j];
        mdensity += H2_1;
        if (H2_1 < 0.0) return 1;
        j++;
        H2_2 = input[j];
        mdensity += H2_2;
        if (H2_2 < 0.0) return 1;
        j++;
        H_1 = input[j];
        mdensity += H_1;
        if (H_1 < 0.0) return 1;
        j++;
        H_2 = input[j];
        mdensity += H_2;
        if (H_2 < 0.0) return 1;
        j++;
        H_m0 = input[j];
        mdensity += H_m0;
        if (H_m0 < 0.0) return 1;
        j++;
        He_1 = input[j];
        mdensity += He_1;
        if (He_1 < 0.0) return 1;
        j++;
        He_2 = input[j];
        mdensity += He_2;
        if (He_2 < 0.0) return 1;
        j++;
        He_3 = input[j];
        mdensity += He_3;
        if (He_3 < 0.0) return 1;
        j++;
        de = input[j];
        if (de < 0.0) return 1;
        j++;
        ge = input[j];
        if (ge < 0.0) return 1;
        j++;
        mdensity *= mh;
        j = i * nchem * nchem;
        Joutput[j] = -k11[i]*H_2 - k12[i]*de - k13[i]*H_1 + k21[i]*pow(H_1, 2) - 2*k23[i]*H2_1;
        j++;
        Joutput[j] = k11[i]*H_2;
        j++;
        Joutput[j] = k11[i]*H_2 + 2*k13[i]*H_1 - 2*k21[i]*pow(H_1, 2) + 4*k23[i]*H2_1;
        j++;
        Joutput[j] = -k11[i]*H_2 + 2*k12[i]*de;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = -H2_1*gloverabel08_gaH2[i]*pow(gloverabel08_gphdl[i], 2)/(pow(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0, 2)*pow(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i], 2)) - H_1*h2formation_h2mcool[i] - gloverabel08_gphdl[i]/(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0);
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = k10[i]*H_1 + k19[i]*H_m0;
        j++;
        Joutput[j] = -k10[i]*H_1 - k18[i]*de - k19[i]*H_m0;
        j++;
        Joutput[j] = -k10[i]*H_1 + 2*k18[i]*de + k19[i]*H_m0;
        j++;
        Joutput[j] = k10[i]*H_1;
        j++;
        Joutput[j] = -k19[i]*H_m0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = -k18[i]*de;
        j++;
        Joutput[j] = 0;
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = k08[i]*H_m0 + k10[i]*H2_2 - k13[i]*H2_1 + 2*k21[i]*H2_1*H_1 + 3*k22[i]*pow(H_1, 2);
        j++;
        Joutput[j] = k09[i]*H_2 - k10[i]*H2_2;
        j++;
        Joutput[j] = -k01[i]*de - k07[i]*de - k08[i]*H_m0 - k09[i]*H_2 - k10[i]*H2_2 + 2*k13[i]*H2_1 + k15[i]*H_m0 - 4*k21[i]*H2_1*H_1 - 6*k22[i]*pow(H_1, 2);
        j++;
        Joutput[j] = k01[i]*de - k09[i]*H_2 + k10[i]*H2_2;
        j++;
        Joutput[j] = k07[i]*de - k08[i]*H_m0 - k15[i]*H_m0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = k01[i]*de - k07[i]*de + k08[i]*H_m0 + k15[i]*H_m0;
        j++;
        Joutput[j] = -H2_1*gloverabel08_gaHI[i]*pow(gloverabel08_gphdl[i], 2)/(pow(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0, 2)*pow(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i], 2)) - H2_1*h2formation_h2mcool[i] + 3*pow(H_1, 2)*h2formation_h2mheat[i] - ceHI_ceHI[i]*de - ciHI_ciHI[i]*de;
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = -k11[i]*H2_1;
        j++;
        Joutput[j] = k09[i]*H_1 + k11[i]*H2_1 + k17[i]*H_m0;
        j++;
        Joutput[j] = k02[i]*de - k09[i]*H_1 + k11[i]*H2_1 + 2*k16[i]*H_m0;
        j++;
        Joutput[j] = -k02[i]*de - k09[i]*H_1 - k11[i]*H2_1 - k16[i]*H_m0 - k17[i]*H_m0;
        j++;
        Joutput[j] = -k16[i]*H_m0 - k17[i]*H_m0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = -k02[i]*de + k17[i]*H_m0;
        j++;
        Joutput[j] = -H2_1*gloverabel08_gaHp[i]*pow(gloverabel08_gphdl[i], 2)/(pow(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0, 2)*pow(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i], 2)) - brem_brem[i]*de - de*reHII_reHII[i];
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = k08[i]*H_1 + k19[i]*H2_2;
        j++;
        Joutput[j] = k17[i]*H_2 - k19[i]*H2_2;
        j++;
        Joutput[j] = -k08[i]*H_1 + k14[i]*de + k15[i]*H_1 + 2*k16[i]*H_2 + k19[i]*H2_2;
        j++;
        Joutput[j] = -k16[i]*H_2 - k17[i]*H_2;
        j++;
        Joutput[j] = -k08[i]*H_1 - k14[i]*de - k15[i]*H_1 - k16[i]*H_2 - k17[i]*H_2 - k19[i]*H2_2;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = k08[i]*H_1 + k14[i]*de + k15[i]*H_1 + k17[i]*H_2;
        j++;
        Joutput[j] = 0;
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = -k03[i]*de;
        j++;
        Joutput[j] = k03[i]*de;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = k03[i]*de;
        j++;
        Joutput[j] = -H2_1*gloverabel08_gaHe[i]*pow(gloverabel08_gphdl[i], 2)/(pow(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0, 2)*pow(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i], 2)) - ciHeI_ciHeI[i]*de;
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = k04[i]*de;
        j++;
        Joutput[j] = -k04[i]*de - k05[i]*de;
        j++;
        Joutput[j] = k05[i]*de;
        j++;
        Joutput[j] = -k04[i]*de + k05[i]*de;
        j++;
        Joutput[j] = -brem_brem[i]*de - ceHeII_ceHeII[i]*de - ceHeI_ceHeI[i]*pow(de, 2) - ciHeII_ciHeII[i]*de - ciHeIS_ciHeIS[i]*pow(de, 2) - de*reHeII1_reHeII1[i] - de*reHeII2_reHeII2[i];
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = k06[i]*de;
        j++;
        Joutput[j] = -k06[i]*de;
        j++;
        Joutput[j] = -k06[i]*de;
        j++;
        Joutput[j] = -4.0*brem_brem[i]*de - de*reHeIII_reHeIII[i];
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = -k12[i]*H2_1;
        j++;
        Joutput[j] = -k18[i]*H2_2;
        j++;
        Joutput[j] = -k01[i]*H_1 + k02[i]*H_2 - k07[i]*H_1 + k14[i]*H_m0 + 2*k18[i]*H2_2;
        j++;
        Joutput[j] = k01[i]*H_1 - k02[i]*H_2 + 2*k12[i]*H2_1;
        j++;
        Joutput[j] = k07[i]*H_1 - k14[i]*H_m0;
        j++;
        Joutput[j] = -k03[i]*He_1 + k04[i]*He_2;
        j++;
        Joutput[j] = k03[i]*He_1 - k04[i]*He_2 - k05[i]*He_2 + k06[i]*He_3;
        j++;
        Joutput[j] = k05[i]*He_2 - k06[i]*He_3;
        j++;
        Joutput[j] = k01[i]*H_1 - k02[i]*H_2 + k03[i]*He_1 - k04[i]*He_2 + k05[i]*He_2 - k06[i]*He_3 - k07[i]*H_1 + k14[i]*H_m0 - k18[i]*H2_2;
        j++;
        Joutput[j] = -H2_1*gloverabel08_gael[i]*pow(gloverabel08_gphdl[i], 2)/(pow(gloverabel08_gphdl[i]/(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i]) + 1.0, 2)*pow(H2_1*gloverabel08_gaH2[i] + H_1*gloverabel08_gaHI[i] + H_2*gloverabel08_gaHp[i] + He_1*gloverabel08_gaHe[i] + de*gloverabel08_gael[i], 2)) - H_1*ceHI_ceHI[i] - H_1*ciHI_ciHI[i] - H_2*reHII_reHII[i] - He_1*ciHeI_ciHeI[i] - He_2*ceHeII_ceHeII[i] - 2*He_2*ceHeI_ceHeI[i]*de - He_2*ciHeII_ciHeII[i] - 2*He_2*ciHeIS_ciHeIS[i]*de - He_2*reHeII1_reHeII1[i] - He_2*reHeII2_reHeII2[i] - He_3*reHeIII_reHeIII[i] - brem_brem[i]*(H_2 + He_2 + 4.0*He_3) - compton_comp[i]*pow(z + 1.0, 4)*(T - 2.73*z - 2.73);
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] *= Tge[i];
        j++;
        Joutput[j] = 0;
        Joutput[j] /= mdensity;
        Joutput[j] *= Tge[i];
        j++;
    }
    return 0;
}

void dgo_primordial_compton_ensure_electron_consistency(double *input, int nstrip, int nchem)
{
    int i, j;
    double H2_1;
    double H2_2;
    double H_1;
    double H_2;
    double H_m0;
    double He_1;
    double He_2;
    double He_3;
    double de;
    double ge;
    double total_e = 0.0;
    int e_indx = 0;
    for (i = 0; i < nstrip; i++) {
        j = i * nchem;
        H2_1 = input[j];
        total_e += H2_1 * 0.0;
        j++;
        H2_2 = input[j];
        total_e += H2_2 * 1.0;
        j++;
        H_1 = input[j];
        total_e += H_1 * 0.0;
        j++;
        H_2 = input[j];
        total_e += H_2 * 1.0;
        j++;
        H_m0 = input[j];
        total_e += H_m0 * -1.0;
        j++;
        He_1 = input[j];
        total_e += He_1 * 0.0;
        j++;
        He_2 = input[j];
        total_e += He_2 * 1.0;
        j++;
        He_3 = input[j];
        total_e += He_3 * 2.0;
        j++;
        de = input[j];
        e_indx = j;
        j++;
        ge = input[j];
        j++;
        input[e_indx] = total_e;
    }
}

static const double unit[NCHEM] = {
    2.0 * 1.67e-24,
    2.0 * 1.67e-24,
    1.00794 * 1.67e-24,
    1.00794 * 1.67e-24,
    1.00794 * 1.67e-24,
    4.002602 * 1.67e-24,
    4.002602 * 1.67e-24,
    4.002602 * 1.67e-24,
    1.0 * 1.67e-24,
    1.0,
};

const dgo_network dgo_primordial_compton_network = {
    "primordial_compton", NCHEM, 9, unit, 0,
    dgo_calculate_rhs_primordial_compton, dgo_calculate_jacobian_primordial_compton,
    dgo_primordial_compton_ensure_electron_consistency,
    alloc_data, free_data, set_z, get_Ts,
};

int dgo_primordial_compton_ntables(void) { return NTAB; }
int dgo_primordial_compton_table_len(int k) { return zdep[k] ? NZ_LEN : NT_LEN; }

/* table k's name in the table bundle (<name>_tables.dgt), so the oracle can
 * order a bundle's tables itself */
static const char *const table_names[NTAB > 0 ? NTAB : 1] = {
    "k01",
    "k02",
    "k03",
    "k04",
    "k05",
    "k06",
    "k07",
    "k08",
    "k09",
    "k10",
    "k11",
    "k12",
    "k13",
    "k14",
    "k15",
    "k16",
    "k17",
    "k18",
    "k19",
    "k21",
    "k22",
    "k23",
    "brem_brem",
    "ceHI_ceHI",
    "ceHeI_ceHeI",
    "ceHeII_ceHeII",
    "ciHI_ciHI",
    "ciHeI_ciHeI",
    "ciHeII_ciHeII",
    "ciHeIS_ciHeIS",
    "compton_comp",
    "gammah_gammah",
    "gloverabel08_gaH2",
    "gloverabel08_gaHI",
    "gloverabel08_gaHe",
    "gloverabel08_gaHp",
    "gloverabel08_gael",
    "gloverabel08_gphdl",
    "gloverabel08_gpldl",
    "h2formation_h2mcool",
    "h2formation_h2mheat",
    "reHII_reHII",
    "reHeII1_reHeII1",
    "reHeII2_reHeII2",
    "reHeIII_reHeIII",
};
const char *dgo_primordial_compton_table_name(int k) { return k >= 0 && k < NTAB ? table_names[k] : 0; }
