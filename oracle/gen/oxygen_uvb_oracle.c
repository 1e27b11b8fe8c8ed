/*
 * ORACLE -- test infrastructure, not part of the product.
 * Generated by oracle/gen_oracle.py for network "oxygen_uvb"; do not edit.
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
#define NCHEM 16
#define NTAB 58
#define NT_LEN 8192
#define NZ_LEN 100
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
} dgo_oxygen_uvb_data;

static const int zdep[NTAB > 0 ? NTAB : 1] = { 0, 1, 0, 0, 1, 0, 1, 0, 0, 0, 1, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 0, 1, 0, 0, 1, 0, 1, 0, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0,  };

static void *alloc_data(const double *const *tables)
{
    int k;
    dgo_oxygen_uvb_data *data = (dgo_oxygen_uvb_data *)calloc(1, sizeof(*data));
    data->bounds[0] = 1.0;
    data->bounds[1] = 10000000000.0;
    data->nbins = NT_LEN - 1;
    data->dbin = (log(data->bounds[1]) - log(data->bounds[0])) / data->nbins;
    data->idbin = 1.0L / data->dbin;
    data->z_bounds[0] = 0.0;
    data->z_bounds[1] = 15.0;
    data->n_zbins = NZ_LEN - 1;
    data->d_zbin = (log(data->z_bounds[1] + 1.0) - log(data->z_bounds[0] + 1.0)) / data->n_zbins;
    data->id_zbin = 1.0L / data->d_zbin;
    for (k = 0; k < NTAB; k++)
        memcpy(data->r[k], tables[k], sizeof(double) * (zdep[k] ? NZ_LEN : NT_LEN));
    return data;
}

static void free_data(void *d) { free(d); }
static void set_z(void *d, double z) { ((dgo_oxygen_uvb_data *)d)->current_z = z; }
static const double *get_Ts(const void *d) { return ((const dgo_oxygen_uvb_data *)d)->Ts; }

void dgo_oxygen_uvb_calculate_temperature(dgo_oxygen_uvb_data *data, double *input,
                                            int nstrip, int nchem)
{
    int i, j;
    double density;
    double kb = 1.3806504e-16;
    double mh = 1.67e-24;
    double gamma = 5.e0/3.e0;
    double gammaH2 = 7.e0/5.e0;
    (void)gammaH2;
    double H_1;
    double H_2;
    double He_1;
    double He_2;
    double He_3;
    double O_1;
    double O_2;
    double O_3;
    double O_4;
    double O_5;
    double O_6;
    double O_7;
    double O_8;
    double O_9;
    double de;
    double ge;
    for (i = 0; i < nstrip; i++) {
        j = i * nchem;
        H_1 = input[j];
        j++;
        H_2 = input[j];
        j++;
        He_1 = input[j];
        j++;
        He_2 = input[j];
        j++;
        He_3 = input[j];
        j++;
        O_1 = input[j];
        j++;
        O_2 = input[j];
        j++;
        O_3 = input[j];
        j++;
        O_4 = input[j];
        j++;
        O_5 = input[j];
        j++;
        O_6 = input[j];
        j++;
        O_7 = input[j];
        j++;
        O_8 = input[j];
        j++;
        O_9 = input[j];
        j++;
        de = input[j];
        j++;
        ge = input[j];
        j++;
        density = 1.0079400000000001*H_1 + 1.0079400000000001*H_2 + 4.0026020000000004*He_1 + 4.0026020000000004*He_2 + 4.0026020000000004*He_3 + 15.9994*O_1 + 15.9994*O_2 + 15.9994*O_3 + 15.9994*O_4 + 15.9994*O_5 + 15.9994*O_6 + 15.9994*O_7 + 15.9994*O_8 + 15.9994*O_9;
        data->Ts[i] = density*ge*mh/(kb*(H_1/(gamma - 1.0) + H_2/(gamma - 1.0) + He_1/(gamma - 1.0) + He_2/(gamma - 1.0) + He_3/(gamma - 1.0) + O_1/(gamma - 1.0) + O_2/(gamma - 1.0) + O_3/(gamma - 1.0) + O_4/(gamma - 1.0) + O_5/(gamma - 1.0) + O_6/(gamma - 1.0) + O_7/(gamma - 1.0) + O_8/(gamma - 1.0) + O_9/(gamma - 1.0) + de/(gamma - 1.0)));
        if (data->Ts[i] < data->bounds[0]) {
            data->Ts[i] = data->bounds[0];
        } else if (data->Ts[i] > data->bounds[1]) {
            data->Ts[i] = data->bounds[1];
        }
        data->logTs[i] = DGO_LOG(data->Ts[i]);
        data->invTs[i] = 1.0 / data->Ts[i];
        data->dTs_ge[i] = density*mh/(kb*(H_1/(gamma - 1.0) + H_2/(gamma - 1.0) + He_1/(gamma - 1.0) + He_2/(gamma - 1.0) + He_3/(gamma - 1.0) + O_1/(gamma - 1.0) + O_2/(gamma - 1.0) + O_3/(gamma - 1.0) + O_4/(gamma - 1.0) + O_5/(gamma - 1.0) + O_6/(gamma - 1.0) + O_7/(gamma - 1.0) + O_8/(gamma - 1.0) + O_9/(gamma - 1.0) + de/(gamma - 1.0)));
    }
}

void dgo_oxygen_uvb_interpolate_rates(dgo_oxygen_uvb_data *data, int nstrip)
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

int dgo_calculate_rhs_oxygen_uvb(double *input, double *rhs, int nstrip, int nchem,
                                   void *sdata)
{
    dgo_oxygen_uvb_data *data = (dgo_oxygen_uvb_data *)sdata;
    int i, j;
    dgo_oxygen_uvb_calculate_temperature(data, input, nstrip, nchem);
    dgo_oxygen_uvb_interpolate_rates(data, nstrip);
    double *H_1_i = data->rs[0];
    double *H_1_pi = data->rs[1];
    double *H_2_r = data->rs[2];
    double *He_1_i = data->rs[3];
    double *He_1_pi = data->rs[4];
    double *He_2_i = data->rs[5];
    double *He_2_pi = data->rs[6];
    double *He_2_r = data->rs[7];
    double *He_3_r = data->rs[8];
    double *O_1_i = data->rs[9];
    double *O_1_pi = data->rs[10];
    double *O_2_i = data->rs[11];
    double *O_2_pi = data->rs[12];
    double *O_2_r = data->rs[13];
    double *O_3_i = data->rs[14];
    double *O_3_pi = data->rs[15];
    double *O_3_r = data->rs[16];
    double *O_4_i = data->rs[17];
    double *O_4_pi = data->rs[18];
    double *O_4_r = data->rs[19];
    double *O_5_i = data->rs[20];
    double *O_5_pi = data->rs[21];
    double *O_5_r = data->rs[22];
    double *O_6_i = data->rs[23];
    double *O_6_pi = data->rs[24];
    double *O_6_r = data->rs[25];
    double *O_7_i = data->rs[26];
    double *O_7_pi = data->rs[27];
    double *O_7_r = data->rs[28];
    double *O_8_i = data->rs[29];
    double *O_8_pi = data->rs[30];
    double *O_8_r = data->rs[31];
    double *O_9_r = data->rs[32];
    double *H_1_c_H_1_c = data->rs[33];
    double *H_1_ph_H_1_ph = data->rs[34];
    double *H_2_c_H_2_c = data->rs[35];
    double *He_1_c_He_1_c = data->rs[36];
    double *He_1_ph_He_1_ph = data->rs[37];
    double *He_2_c_He_2_c = data->rs[38];
    double *He_2_ph_He_2_ph = data->rs[39];
    double *He_3_c_He_3_c = data->rs[40];
    double *O_1_c_O_1_c = data->rs[41];
    double *O_1_ph_O_1_ph = data->rs[42];
    double *O_2_c_O_2_c = data->rs[43];
    double *O_2_ph_O_2_ph = data->rs[44];
    double *O_3_c_O_3_c = data->rs[45];
    double *O_3_ph_O_3_ph = data->rs[46];
    double *O_4_c_O_4_c = data->rs[47];
    double *O_4_ph_O_4_ph = data->rs[48];
    double *O_5_c_O_5_c = data->rs[49];
    double *O_5_ph_O_5_ph = data->rs[50];
    double *O_6_c_O_6_c = data->rs[51];
    double *O_6_ph_O_6_ph = data->rs[52];
    double *O_7_c_O_7_c = data->rs[53];
    double *O_7_ph_O_7_ph = data->rs[54];
    double *O_8_c_O_8_c = data->rs[55];
    double *O_8_ph_O_8_ph = data->rs[56];
    double *O_9_c_O_9_c = data->rs[57];
    double H_1;
    double H_2;
    double He_1;
    double He_2;
    double He_3;
    double O_1;
    double O_2;
    double O_3;
    double O_4;
    double O_5;
    double O_6;
    double O_7;
    double O_8;
    double O_9;
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
        H_1 = input[j];
        mdensity += H_1;
        if (H_1 < 0.0) return 1;
        j++;
        H_2 = input[j];
        mdensity += H_2;
        if (H_2 < 0.0) return 1;
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
        O_1 = input[j];
        mdensity += O_1;
        if (O_1 < 0.0) return 1;
        j++;
        O_2 = input[j];
        mdensity += O_2;
        if (O_2 < 0.0) return 1;
        j++;
        O_3 = input[j];
        mdensity += O_3;
        if (O_3 < 0.0) return 1;
        j++;
        O_4 = input[j];
        mdensity += O_4;
        if (O_4 < 0.0) return 1;
        j++;
        O_5 = input[j];
        mdensity += O_5;
        if (O_5 < 0.0) return 1;
        j++;
        O_6 = input[j];
        mdensity += O_6;
        if (O_6 < 0.0) return 1;
        j++;
        O_7 = input[j];
        mdensity += O_7;
        if (O_7 < 0.0) return 1;
        j++;
        O_8 = input[j];
        mdensity += O_8;
        if (O_8 < 0.0) return 1;
        j++;
        O_9 = input[j];
        mdensity += O_9;
        if (O_9 < 0.0) return 1;
        j++;
        de = input[j];
        if (de < 0.0) return 1;
        j++;
        ge = input[j];
        if (ge < 0.0) return 1;
        j++;
        mdensity *= mh;
        j = i * nchem;
        rhs[j] = -H_1_i[i]*H_1*de - H_1_pi[i]*H_1 + H_2_r[i]*H_2*de;
        j++;
        rhs[j] = H_1_i[i]*H_1*de + H_1_pi[i]*H_1 - H_2_r[i]*H_2*de;
        j++;
        rhs[j] = -He_1_i[i]*He_1*de - He_1_pi[i]*He_1 + He_2_r[i]*He_2*de;
        j++;
        rhs[j] = He_1_i[i]*He_1*de + He_1_pi[i]*He_1 - He_2_i[i]*He_2*de - He_2_pi[i]*He_2 - He_2_r[i]*He_2*de + He_3_r[i]*He_3*de;
        j++;
        rhs[j] = He_2_i[i]*He_2*de + He_2_pi[i]*He_2 - He_3_r[i]*He_3*de;
        j++;
        rhs[j] = -O_1_i[i]*O_1*de - O_1_pi[i]*O_1 + O_2_r[i]*O_2*de;
        j++;
        rhs[j] = O_1_i[i]*O_1*de + O_1_pi[i]*O_1 - O_2_i[i]*O_2*de - O_2_pi[i]*O_2 - O_2_r[i]*O_2*de + O_3_r[i]*O_3*de;
        j++;
        rhs[j] = O_2_i[i]*O_2*de + O_2_pi[i]*O_2 - O_3_i[i]*O_3*de - O_3_pi[i]*O_3 - O_3_r[i]*O_3*de + O_4_r[i]*O_4*de;
        j++;
        rhs[j] = O_3_i[i]*O_3*de + O_3_pi[i]*O_3 - O_4_i[i]*O_4*de - O_4_pi[i]*O_4 - O_4_r[i]*O_4*de + O_5_r[i]*O_5*de;
        j++;
        rhs[j] = O_4_i[i]*O_4*de + O_4_pi[i]*O_4 - O_5_i[i]*O_5*de - O_5_pi[i]*O_5 - O_5_r[i]*O_5*de + O_6_r[i]*O_6*de;
        j++;
        rhs[j] = O_5_i[i]*O_5*de + O_5_pi[i]*O_5 - O_6_i[i]*O_6*de - O_6_pi[i]*O_6 - O_6_r[i]*O_6*de + O_7_r[i]*O_7*de;
        j++;
        rhs[j] = O_6_i[i]*O_6*de + O_6_pi[i]*O_6 - O_7_i[i]*O_7*de - O_7_pi[i]*O_7 - O_7_r[i]*O_7*de + O_8_r[i]*O_8*de;
        j++;
        rhs[j] = O_7_i[i]*O_7*de + O_7_pi[i]*O_7 - O_8_i[i]*O_8*de - O_8_pi[i]*O_8 - O_8_r[i]*O_8*de + O_9_r[i]*O_9*de;
        j++;
        rhs[j] = O_8_i[i]*O_8*de + O_8_pi[i]*O_8 - O_9_r[i]*O_9*de;
        j++;
        rhs[j] = H_1_i[i]*H_1*de + H_1_pi[i]*H_1 - H_2_r[i]*H_2*de + He_1_i[i]*He_1*de + He_1_pi[i]*He_1 + He_2_i[i]*He_2*de + He_2_pi[i]*He_2 - He_2_r[i]*He_2*de - He_3_r[i]*He_3*de + O_1_i[i]*O_1*de + O_1_pi[i]*O_1 + O_2_i[i]*O_2*de + O_2_pi[i]*O_2 - O_2_r[i]*O_2*de + O_3_i[i]*O_3*de + O_3_pi[i]*O_3 - O_3_r[i]*O_3*de + O_4_i[i]*O_4*de + O_4_pi[i]*O_4 - O_4_r[i]*O_4*de + O_5_i[i]*O_5*de + O_5_pi[i]*O_5 - O_5_r[i]*O_5*de + O_6_i[i]*O_6*de + O_6_pi[i]*O_6 - O_6_r[i]*O_6*de + O_7_i[i]*O_7*de + O_7_pi[i]*O_7 - O_7_r[i]*O_7*de + O_8_i[i]*O_8*de + O_8_pi[i]*O_8 - O_8_r[i]*O_8*de - O_9_r[i]*O_9*de;
        j++;
        rhs[j] = -H_1*H_1_c_H_1_c[i]*de + H_1*H_1_ph_H_1_ph[i] - H_2*H_2_c_H_2_c[i]*de - He_1*He_1_c_He_1_c[i]*de + He_1*He_1_ph_He_1_ph[i] - He_2*He_2_c_He_2_c[i]*de + He_2*He_2_ph_He_2_ph[i] - He_3*He_3_c_He_3_c[i]*de - O_1*O_1_c_O_1_c[i]*de + O_1*O_1_ph_O_1_ph[i] - O_2*O_2_c_O_2_c[i]*de + O_2*O_2_ph_O_2_ph[i] - O_3*O_3_c_O_3_c[i]*de + O_3*O_3_ph_O_3_ph[i] - O_4*O_4_c_O_4_c[i]*de + O_4*O_4_ph_O_4_ph[i] - O_5*O_5_c_O_5_c[i]*de + O_5*O_5_ph_O_5_ph[i] - O_6*O_6_c_O_6_c[i]*de + O_6*O_6_ph_O_6_ph[i] - O_7*O_7_c_O_7_c[i]*de + O_7*O_7_ph_O_7_ph[i] - O_8*O_8_c_O_8_c[i]*de + O_8*O_8_ph_O_8_ph[i] - O_9*O_9_c_O_9_c[i]*de;
        rhs[j] /= mdensity;
        j++;
    }
    return 0;
}

int dgo_calculate_jacobian_oxygen_uvb(double *input, double *Joutput, int nstrip,
                                        int nchem, void *sdata)
{
    dgo_oxygen_uvb_data *data = (dgo_oxygen_uvb_data *)sdata;
    int i, j;
    double *Tge = data->dTs_ge;
    double *H_1_i = data->rs[0];
    double *H_1_pi = data->rs[1];
    double *H_2_r = data->rs[2];
    double *He_1_i = data->rs[3];
    double *He_1_pi = data->rs[4];
    double *He_2_i = data->rs[5];
    double *He_2_pi = data->rs[6];
    double *He_2_r = data->rs[7];
    double *He_3_r = data->rs[8];
    double *O_1_i = data->rs[9];
    double *O_1_pi = data->rs[10];
    double *O_2_i = data->rs[11];
    double *O_2_pi = data->rs[12];
    double *O_2_r = data->rs[13];
    double *O_3_i = data->rs[14];
    double *O_3_pi = data->rs[15];
    double *O_3_r = data->rs[16];
    double *O_4_i = data->rs[17];
    double *O_4_pi = data->rs[18];
    double *O_4_r = data->rs[19];
    double *O_5_i = data->rs[20];
    double *O_5_pi = data->rs[21];
    double *O_5_r = data->rs[22];
    double *O_6_i = data->rs[23];
    double *O_6_pi = data->rs[24];
    double *O_6_r = data->rs[25];
    double *O_7_i = data->rs[26];
    double *O_7_pi = data->rs[27];
    double *O_7_r = data->rs[28];
    double *O_8_i = data->rs[29];
    double *O_8_pi = data->rs[30];
    double *O_8_r = data->rs[31];
    double *O_9_r = data->rs[32];
    double *H_1_c_H_1_c = data->rs[33];
    double *H_1_ph_H_1_ph = data->rs[34];
    double *H_2_c_H_2_c = data->rs[35];
    double *He_1_c_He_1_c = data->rs[36];
    double *He_1_ph_He_1_ph = data->rs[37];
    double *He_2_c_He_2_c = data->rs[38];
    double *He_2_ph_He_2_ph = data->rs[39];
    double *He_3_c_He_3_c = data->rs[40];
    double *O_1_c_O_1_c = data->rs[41];
    double *O_1_ph_O_1_ph = data->rs[42];
    double *O_2_c_O_2_c = data->rs[43];
    double *O_2_ph_O_2_ph = data->rs[44];
    double *O_3_c_O_3_c = data->rs[45];
    double *O_3_ph_O_3_ph = data->rs[46];
    double *O_4_c_O_4_c = data->rs[47];
    double *O_4_ph_O_4_ph = data->rs[48];
    double *O_5_c_O_5_c = data->rs[49];
    double *O_5_ph_O_5_ph = data->rs[50];
    double *O_6_c_O_6_c = data->rs[51];
    double *O_6_ph_O_6_ph = data->rs[52];
    double *O_7_c_O_7_c = data->rs[53];
    double *O_7_ph_O_7_ph = data->rs[54];
    double *O_8_c_O_8_c = data->rs[55];
    double *O_8_ph_O_8_ph = data->rs[56];
    double *O_9_c_O_9_c = data->rs[57];
    double H_1;
    double H_2;
    double He_1;
    double He_2;
    double He_3;
    double O_1;
    double O_2;
    double O_3;
    double O_4;
    double O_5;
    double O_6;
    double O_7;
    double O_8;
    double O_9;
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
        H_1 = input[j];
        mdensity += H_1;
        if (H_1 < 0.0) return 1;
        j++;
        H_2 = input[j];
        mdensity += H_2;
        if (H_2 < 0.0) return 1;
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
        O_1 = input[j];
        mdensity += O_1;
        if (O_1 < 0.0) return 1;
        j++;
        O_2 = input[j];
        mdensity += O_2;
        if (O_2 < 0.0) return 1;
        j++;
        O_3 = input[j];
        mdensity += O_3;
        if (O_3 < 0.0) return 1;
        j++;
        O_4 = input[j];
        mdensity += O_4;
        if (O_4 < 0.0) return 1;
        j++;
        O_5 = input[j];
        mdensity += O_5;
        if (O_5 < 0.0) return 1;
        j++;
        O_6 = input[j];
        mdensity += O_6;
        if (O_6 < 0.0) return 1;
        j++;
        O_7 = input[j];
        mdensity += O_7;
        if (O_7 < 0.0) return 1;
        j++;
        O_8 = input[j];
        mdensity += O_8;
        if (O_8 < 0.0) return 1;
        j++;
        O_9 = input[j];
        mdensity += O_9;
        if (O_9 < 0.0) return 1;
        j++;
        de = input[j];
        if (de < 0.0) return 1;
        j++;
        ge = input[j];
        if (ge < 0.0) return 1;
        j++;
        mdensity *= mh;
        j = i * nchem * nchem;
        Joutput[j] = -H_1_i[i]*de - H_1_pi[i];
        j++;
        Joutput[j] = H_1_i[i]*de + H_1_pi[i];
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
        Joutput[j] = H_1_i[i]*de + H_1_pi[i];
        j++;
        Joutput[j] = -H_1_c_H_1_c[i]*de + H_1_ph_H_1_ph[i];
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = H_2_r[i]*de;
        j++;
        Joutput[j] = -H_2_r[i]*de;
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
        Joutput[j] = -H_2_r[i]*de;
        j++;
        Joutput[j] = -H_2_c_H_2_c[i]*de;
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = -He_1_i[i]*de - He_1_pi[i];
        j++;
        Joutput[j] = He_1_i[i]*de + He_1_pi[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = He_1_i[i]*de + He_1_pi[i];
        j++;
        Joutput[j] = -He_1_c_He_1_c[i]*de + He_1_ph_He_1_ph[i];
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = He_2_r[i]*de;
        j++;
        Joutput[j] = -He_2_i[i]*de - He_2_pi[i] - He_2_r[i]*de;
        j++;
        Joutput[j] = He_2_i[i]*de + He_2_pi[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = He_2_i[i]*de + He_2_pi[i] - He_2_r[i]*de;
        j++;
        Joutput[j] = -He_2_c_He_2_c[i]*de + He_2_ph_He_2_ph[i];
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = He_3_r[i]*de;
        j++;
        Joutput[j] = -He_3_r[i]*de;
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = -He_3_r[i]*de;
        j++;
        Joutput[j] = -He_3_c_He_3_c[i]*de;
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
        Joutput[j] = -O_1_i[i]*de - O_1_pi[i];
        j++;
        Joutput[j] = O_1_i[i]*de + O_1_pi[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_1_i[i]*de + O_1_pi[i];
        j++;
        Joutput[j] = -O_1_c_O_1_c[i]*de + O_1_ph_O_1_ph[i];
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
        Joutput[j] = O_2_r[i]*de;
        j++;
        Joutput[j] = -O_2_i[i]*de - O_2_pi[i] - O_2_r[i]*de;
        j++;
        Joutput[j] = O_2_i[i]*de + O_2_pi[i];
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
        Joutput[j] = O_2_i[i]*de + O_2_pi[i] - O_2_r[i]*de;
        j++;
        Joutput[j] = -O_2_c_O_2_c[i]*de + O_2_ph_O_2_ph[i];
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
        Joutput[j] = O_3_r[i]*de;
        j++;
        Joutput[j] = -O_3_i[i]*de - O_3_pi[i] - O_3_r[i]*de;
        j++;
        Joutput[j] = O_3_i[i]*de + O_3_pi[i];
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
        Joutput[j] = O_3_i[i]*de + O_3_pi[i] - O_3_r[i]*de;
        j++;
        Joutput[j] = -O_3_c_O_3_c[i]*de + O_3_ph_O_3_ph[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_4_r[i]*de;
        j++;
        Joutput[j] = -O_4_i[i]*de - O_4_pi[i] - O_4_r[i]*de;
        j++;
        Joutput[j] = O_4_i[i]*de + O_4_pi[i];
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_4_i[i]*de + O_4_pi[i] - O_4_r[i]*de;
        j++;
        Joutput[j] = -O_4_c_O_4_c[i]*de + O_4_ph_O_4_ph[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_5_r[i]*de;
        j++;
        Joutput[j] = -O_5_i[i]*de - O_5_pi[i] - O_5_r[i]*de;
        j++;
        Joutput[j] = O_5_i[i]*de + O_5_pi[i];
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_5_i[i]*de + O_5_pi[i] - O_5_r[i]*de;
        j++;
        Joutput[j] = -O_5_c_O_5_c[i]*de + O_5_ph_O_5_ph[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_6_r[i]*de;
        j++;
        Joutput[j] = -O_6_i[i]*de - O_6_pi[i] - O_6_r[i]*de;
        j++;
        Joutput[j] = O_6_i[i]*de + O_6_pi[i];
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_6_i[i]*de + O_6_pi[i] - O_6_r[i]*de;
        j++;
        Joutput[j] = -O_6_c_O_6_c[i]*de + O_6_ph_O_6_ph[i];
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
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_7_r[i]*de;
        j++;
        Joutput[j] = -O_7_i[i]*de - O_7_pi[i] - O_7_r[i]*de;
        j++;
        Joutput[j] = O_7_i[i]*de + O_7_pi[i];
        j++;
        Joutput[j] = 0;
        j++;
        Joutput[j] = O_7_i[i]*de + O_7_pi[i] - O_7_r[i]*de;
        j++;
        Joutput[j] = -O_7_c_O_7_c[i]*de + O_7_ph_O_7_ph[i];
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
        Joutput[j] = O_8_r[i]*de;
        j++;
        Joutput[j] = -O_8_i[i]*de - O_8_pi[i] - O_8_r[i]*de;
        j++;
        Joutput[j] = O_8_i[i]*de + O_8_pi[i];
        j++;
        Joutput[j] = O_8_i[i]*de + O_8_pi[i] - O_8_r[i]*de;
        j++;
        Joutput[j] = -O_8_c_O_8_c[i]*de + O_8_ph_O_8_ph[i];
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
        Joutput[j] = O_9_r[i]*de;
        j++;
        Joutput[j] = -O_9_r[i]*de;
        j++;
        Joutput[j] = -O_9_r[i]*de;
        j++;
        Joutput[j] = -O_9_c_O_9_c[i]*de;
        Joutput[j] /= mdensity;
        j++;
        Joutput[j] = -H_1_i[i]*H_1 + H_2_r[i]*H_2;
        j++;
        Joutput[j] = H_1_i[i]*H_1 - H_2_r[i]*H_2;
        j++;
        Joutput[j] = -He_1_i[i]*He_1 + He_2_r[i]*He_2;
        j++;
        Joutput[j] = He_1_i[i]*He_1 - He_2_i[i]*He_2 - He_2_r[i]*He_2 + He_3_r[i]*He_3;
        j++;
        Joutput[j] = He_2_i[i]*He_2 - He_3_r[i]*He_3;
        j++;
        Joutput[j] = -O_1_i[i]*O_1 + O_2_r[i]*O_2;
        j++;
        Joutput[j] = O_1_i[i]*O_1 - O_2_i[i]*O_2 - O_2_r[i]*O_2 + O_3_r[i]*O_3;
        j++;
        Joutput[j] = O_2_i[i]*O_2 - O_3_i[i]*O_3 - O_3_r[i]*O_3 + O_4_r[i]*O_4;
        j++;
        Joutput[j] = O_3_i[i]*O_3 - O_4_i[i]*O_4 - O_4_r[i]*O_4 + O_5_r[i]*O_5;
        j++;
        Joutput[j] = O_4_i[i]*O_4 - O_5_i[i]*O_5 - O_5_r[i]*O_5 + O_6_r[i]*O_6;
        j++;
        Joutput[j] = O_5_i[i]*O_5 - O_6_i[i]*O_6 - O_6_r[i]*O_6 + O_7_r[i]*O_7;
        j++;
        Joutput[j] = O_6_i[i]*O_6 - O_7_i[i]*O_7 - O_7_r[i]*O_7 + O_8_r[i]*O_8;
        j++;
        Joutput[j] = O_7_i[i]*O_7 - O_8_i[i]*O_8 - O_8_r[i]*O_8 + O_9_r[i]*O_9;
        j++;
        Joutput[j] = O_8_i[i]*O_8 - O_9_r[i]*O_9;
        j++;
        Joutput[j] = H_1_i[i]*H_1 - H_2_r[i]*H_2 + He_1_i[i]*He_1 + He_2_i[i]*He_2 - He_2_r[i]*He_2 - He_3_r[i]*He_3 + O_1_i[i]*O_1 + O_2_i[i]*O_2 - O_2_r[i]*O_2 + O_3_i[i]*O_3 - O_3_r[i]*O_3 + O_4_i[i]*O_4 - O_4_r[i]*O_4 + O_5_i[i]*O_5 - O_5_r[i]*O_5 + O_6_i[i]*O_6 - O_6_r[i]*O_6 + O_7_i[i]*O_7 - O_7_r[i]*O_7 + O_8_i[i]*O_8 - O_8_r[i]*O_8 - O_9_r[i]*O_9;
        j++;
        Joutput[j] = -H_1*H_1_c_H_1_c[i] - H_2*H_2_c_H_2_c[i] - He_1*He_1_c_He_1_c[i] - He_2*He_2_c_He_2_c[i] - He_3*He_3_c_He_3_c[i] - O_1*O_1_c_O_1_c[i] - O_2*O_2_c_O_2_c[i] - O_3*O_3_c_O_3_c[i] - O_4*O_4_c_O_4_c[i] - O_5*O_5_c_O_5_c[i] - O_6*O_6_c_O_6_c[i] - O_7*O_7_c_O_7_c[i] - O_8*O_8_c_O_8_c[i] - O_9*O_9_c_O_9_c[i];
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

void dgo_oxygen_uvb_ensure_electron_consistency(double *input, int nstrip, int nchem)
{
    int i, j;
    double H_1;
    double H_2;
    double He_1;
    double He_2;
    double He_3;
    double O_1;
    double O_2;
    double O_3;
    double O_4;
    double O_5;
    double O_6;
    double O_7;
    double O_8;
    double O_9;
    double de;
    double ge;
    double total_e = 0.0;
    int e_indx = 0;
    for (i = 0; i < nstrip; i++) {
        j = i * nchem;
        H_1 = input[j];
        total_e += H_1 * 0;
        j++;
        H_2 = input[j];
        total_e += H_2 * 1;
        j++;
        He_1 = input[j];
        total_e += He_1 * 0;
        j++;
        He_2 = input[j];
        total_e += He_2 * 1;
        j++;
        He_3 = input[j];
        total_e += He_3 * 2;
        j++;
        O_1 = input[j];
        total_e += O_1 * 0;
        j++;
        O_2 = input[j];
        total_e += O_2 * 1;
        j++;
        O_3 = input[j];
        total_e += O_3 * 2;
        j++;
        O_4 = input[j];
        total_e += O_4 * 3;
        j++;
        O_5 = input[j];
        total_e += O_5 * 4;
        j++;
        O_6 = input[j];
        total_e += O_6 * 5;
        j++;
        O_7 = input[j];
        total_e += O_7 * 6;
        j++;
        O_8 = input[j];
        total_e += O_8 * 7;
        j++;
        O_9 = input[j];
        total_e += O_9 * 8;
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
    1.00794 * 1.67e-24,
    1.00794 * 1.67e-24,
    4.002602 * 1.67e-24,
    4.002602 * 1.67e-24,
    4.002602 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    15.9994 * 1.67e-24,
    1.0 * 1.67e-24,
    1.0,
};

const dgo_network dgo_oxygen_uvb_network = {
    "oxygen_uvb", NCHEM, 15, unit, 0,
    dgo_calculate_rhs_oxygen_uvb, dgo_calculate_jacobian_oxygen_uvb,
    dgo_oxygen_uvb_ensure_electron_consistency,
    alloc_data, free_data, set_z, get_Ts,
};

int dgo_oxygen_uvb_ntables(void) { return NTAB; }
int dgo_oxygen_uvb_table_len(int k) { return zdep[k] ? NZ_LEN : NT_LEN; }

/* table k's name in the table bundle (<name>_tables.dgt), so the oracle can
 * order a bundle's tables itself */
static const char *const table_names[NTAB > 0 ? NTAB : 1] = {
    "H_1_i",
    "H_1_pi",
    "H_2_r",
    "He_1_i",
    "He_1_pi",
    "He_2_i",
    "He_2_pi",
    "He_2_r",
    "He_3_r",
    "O_1_i",
    "O_1_pi",
    "O_2_i",
    "O_2_pi",
    "O_2_r",
    "O_3_i",
    "O_3_pi",
    "O_3_r",
    "O_4_i",
    "O_4_pi",
    "O_4_r",
    "O_5_i",
    "O_5_pi",
    "O_5_r",
    "O_6_i",
    "O_6_pi",
    "O_6_r",
    "O_7_i",
    "O_7_pi",
    "O_7_r",
    "O_8_i",
    "O_8_pi",
    "O_8_r",
    "O_9_r",
    "H_1_c_H_1_c",
    "H_1_ph_H_1_ph",
    "H_2_c_H_2_c",
    "He_1_c_He_1_c",
    "He_1_ph_He_1_ph",
    "He_2_c_He_2_c",
    "He_2_ph_He_2_ph",
    "He_3_c_He_3_c",
    "O_1_c_O_1_c",
    "O_1_ph_O_1_ph",
    "O_2_c_O_2_c",
    "O_2_ph_O_2_ph",
    "O_3_c_O_3_c",
    "O_3_ph_O_3_ph",
    "O_4_c_O_4_c",
    "O_4_ph_O_4_ph",
    "O_5_c_O_5_c",
    "O_5_ph_O_5_ph",
    "O_6_c_O_6_c",
    "O_6_ph_O_6_ph",
    "O_7_c_O_7_c",
    "O_7_ph_O_7_ph",
    "O_8_c_O_8_c",
    "O_8_ph_O_8_ph",
    "O_9_c_O_9_c",
};
const char *dgo_oxygen_uvb_table_name(int k) { return k >= 0 && k < NTAB ? table_names[k] : 0; }
