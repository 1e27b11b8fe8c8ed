/*
 * ORACLE -- test infrastructure, not part of the product.  See be_oracle.h.
 *
 * Restates, in plain C with the same IEEE operation sequence:
 *   BE_chem_solve        dengo/solvers/BE_chem_solve.C:79-241
 *   BE_Resid_Fun         dengo/solvers/BE_chem_solve.C:246-275
 *   BE_Resid_Jac         dengo/solvers/BE_chem_solve.C:280-321
 *   Gauss_Elim           dengo/solvers/BE_chem_solve.C:330-382
 *   dengo_evolve_<name>  dengo/templates/rates_and_rate_tables.C.template:149-274
 *   run_<name>           dengo/templates/rates_and_rate_tables_run.pyx.template:114-205
 * Diagnostic prints of the reference are omitted (they have no effect on
 * results).
 */
#include "be_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define DGO_MIN(A, B) ((A) < (B) ? (A) : (B))

dgo_config dgo_default_config(void)
{
    dgo_config c;
    c.max_sweeps = 10;
    c.max_substeps = 50000;
    c.dt_ratio_floor = 1e-15;
    c.floor_value = 1e-25;
    return c;
}

/* BE_chem_solve.C:246-275 -- g(u) = u - u0 - dt*f(u) in scaled variables. */
static int resid_fun(dgo_rhs_f f, double *u, double *u0, double *gu, double dt,
                     int nstrip, int nchem, const double *scaling,
                     const double *inv_scaling, void *sdata)
{
    int i, n = nstrip * nchem;
    for (i = 0; i < n; i++) u[i] *= scaling[i];
    if (f(u, gu, nstrip, nchem, sdata) != 0) return 1;
    for (i = 0; i < n; i++) u[i] *= inv_scaling[i];
    for (i = 0; i < n; i++) gu[i] *= inv_scaling[i];
    for (i = 0; i < n; i++) gu[i] = u[i] - u0[i] - dt * gu[i];
    return 0;
}

/* BE_chem_solve.C:280-321 -- scaled I - dt*J, column-major per cell. */
static int resid_jac(dgo_jac_f J, double *u, double *Ju, double dt, int nstrip,
                     int nchem, const double *scaling, const double *inv_scaling,
                     void *sdata)
{
    int ix, ivar, jvar, i, n = nstrip * nchem;
    for (i = 0; i < n; i++) u[i] *= scaling[i];
    if (J(u, Ju, nstrip, nchem, sdata) != 0) return 1;
    for (i = 0; i < n; i++) u[i] *= inv_scaling[i];
    for (ix = 0; ix < nstrip; ix++)
        for (jvar = 0; jvar < nchem; jvar++)
            for (ivar = 0; ivar < nchem; ivar++)
                Ju[(ix * nchem + jvar) * nchem + ivar] *= inv_scaling[ix * nchem + ivar];
    for (ix = 0; ix < nstrip; ix++)
        for (ivar = 0; ivar < nchem; ivar++)
            for (jvar = 0; jvar < nchem; jvar++)
                Ju[(ix * nchem + jvar) * nchem + ivar] *= scaling[ix * nchem + jvar];
    for (ix = 0; ix < nstrip * nchem * nchem; ix++) Ju[ix] = -dt * Ju[ix];
    for (ix = 0; ix < nstrip; ix++)
        for (ivar = 0; ivar < nchem; ivar++)
            Ju[ix * nchem * nchem + ivar * nchem + ivar] += 1.0;
    return 0;
}

/* BE_chem_solve.C:329-382 -- partial pivoting; A column-major, A(i,j)=A[j*n+i]. */
#define A_(i, j) A[(j) * n + (i)]
int dgo_Gauss_Elim(double *A, double *x, double *b, int n)
{
    int i, j, k, p;
    double dtmp;
    for (i = 0; i < n; i++) x[i] = b[i];
    for (k = 0; k < n - 1; k++) {
        p = k;
        for (i = k + 1; i < n; i++)
            if (fabs(A_(i, k)) > fabs(A_(p, k))) p = i;
        for (j = k; j < n; j++) {
            dtmp = A_(k, j);
            A_(k, j) = A_(p, j);
            A_(p, j) = dtmp;
        }
        dtmp = x[k];
        x[k] = x[p];
        x[p] = dtmp;
        for (i = k + 1; i < n; i++) A_(i, k) /= A_(k, k);
        for (j = k + 1; j < n; j++)
            for (i = k + 1; i < n; i++) A_(i, j) -= A_(i, k) * A_(k, j);
        for (i = k + 1; i < n; i++) x[i] -= A_(i, k) * x[k];
    }
    for (i = n - 1; i >= 0; i--) {
        for (j = i + 1; j < n; j++) x[i] -= A_(i, j) * x[j];
        x[i] /= A_(i, i);
    }
    return 0;
}
#undef A_

/* BE_chem_solve.C:79-241 */
int dgo_BE_chem_solve(dgo_rhs_f f, dgo_jac_f J, double *u, double dt,
                      double *rtol, double *atol, int nstrip, int nchem,
                      double *scaling, void *sdata, double *u0, double *s,
                      double *gu, double *Ju, int max_sweeps, long long *sweeps)
{
    int i, ix, isweep, ioff, unsolved = 0, n = nstrip * nchem;
    const double lam = 1.0;
    double *inv_scaling = (double *)malloc(sizeof(double) * n);

    for (i = 0; i < n; i++) inv_scaling[i] = 1.0 / scaling[i];
    for (i = 0; i < n; i++) u[i] *= inv_scaling[i];
    for (i = 0; i < n; i++) atol[i] *= inv_scaling[i];
    for (i = 0; i < n; i++) u0[i] = u[i];
    for (i = 0; i < nchem; i++) s[i] = 0.0;
    for (i = 0; i < n; i++) gu[i] = 0.0;
    for (i = 0; i < n * nchem; i++) Ju[i] = 0.0;

    for (isweep = 0; isweep < max_sweeps; isweep++) {
        if (sweeps) (*sweeps)++;
        if (resid_fun(f, u, u0, gu, dt, nstrip, nchem, scaling, inv_scaling, sdata) != 0 ||
            resid_jac(J, u, Ju, dt, nstrip, nchem, scaling, inv_scaling, sdata) != 0) {
            for (i = 0; i < n; i++) u[i] *= scaling[i];
            for (i = 0; i < n; i++) atol[i] *= scaling[i];
            free(inv_scaling);
            return 1;
        }
        unsolved = 0;
        for (ix = 0; ix < nstrip; ix++) {
            ioff = ix * nchem;
            dgo_Gauss_Elim(&Ju[ix * nchem * nchem], s, &gu[ioff], nchem);
            for (i = 0; i < nchem; i++) u[ioff + i] -= lam * s[i];
            for (i = 0; i < nchem; i++) {
                if (fabs(s[i]) > (atol[ioff + i] + rtol[ioff + i] * fabs(u[ioff + i]))) {
                    unsolved = 1;
                    break;
                }
                if (u[ioff + i] != u[ioff + i]) { /* NaN */
                    for (i = 0; i < n; i++) u[i] *= scaling[i];
                    for (i = 0; i < n; i++) atol[i] *= scaling[i];
                    free(inv_scaling);
                    return 1;
                }
            }
        }
        if (!unsolved) break;
    }
    free(inv_scaling);
    for (i = 0; i < n; i++) u[i] *= scaling[i];
    for (i = 0; i < n; i++) atol[i] *= scaling[i];
    return unsolved ? 1 : 0;
}

static dgo_intermediate_f dgo_hook;
static void *dgo_hook_ctx;

void dgo_set_intermediate_hook(dgo_intermediate_f f, void *ctx)
{
    dgo_hook = f;
    dgo_hook_ctx = ctx;
}

/* rates_and_rate_tables.C.template:149-274 */
double dgo_evolve(const dgo_network *net, void *data, double dtf, double *dtp,
                  double z, double *input, double *rtol, double *atol,
                  long long dims, const dgo_config *cfg, dgo_stats *st)
{
    const int N = net->nchem;
    const long long n = dims * N;
    long long i, c;
    int j;
    double dt = *dtp;

    if (!net->input_is_number) {
        for (c = 0; c < dims; c++)
            for (j = 0; j < N; j++) {
                if (j == net->ige) continue;
                input[c * N + j] /= net->unit[j];
                atol[c * N + j] /= net->unit[j];
            }
    }
    net->electrons(input, (int)dims, N);

    if (dt < 0) dt = dtf / 1e5;
    net->set_z(data, z);
    int siter = 0;
    double ttot = 0;
    double *scale = (double *)malloc(sizeof(double) * n);
    double *prev = (double *)malloc(sizeof(double) * n);
    double *u0 = (double *)malloc(sizeof(double) * n);
    double *s = (double *)malloc(sizeof(double) * N);
    double *gu = (double *)malloc(sizeof(double) * n);
    double *Ju = (double *)malloc(sizeof(double) * n * N);
    for (i = 0; i < n; i++) scale[i] = input[i];
    for (i = 0; i < n; i++) prev[i] = input[i];
    const double floor_value = cfg->floor_value;
    int status = 0;

    while (ttot < dtf) {
        int rv = dgo_BE_chem_solve(net->rhs, net->jac, input, dt, rtol, atol, (int)dims,
                                   N, scale, data, u0, s, gu, Ju, cfg->max_sweeps,
                                   st ? &st->sweeps : NULL);
        for (i = 0; i < n; i++) {
            if (input[i] < 0) {
                rv = 1;
                break;
            }
        }
        if (rv == 0) {
            if (siter == cfg->max_substeps) {
                status = 1;
                break;
            }
            siter++;
            if (st) st->substeps_ok++;
            ttot += dt;
            dt = DGO_MIN(dt * 1.1, dtf - ttot);
            /* C.template:212-241: the intermediate file holds prev (not yet
             * updated), data->Ts, ttot and dt */
            if (dgo_hook) dgo_hook(dgo_hook_ctx, siter, prev, net->Ts(data), dims, N, ttot, dt);
            for (i = 0; i < n; i++) prev[i] = input[i];
            for (i = 0; i < n; i++)
                if (input[i] < floor_value) input[i] = floor_value;
        } else {
            if (st) st->substeps_fail++;
            dt /= 2.0;
            for (i = 0; i < n; i++) input[i] = prev[i];
            if (dt / dtf < cfg->dt_ratio_floor) {
                status = 2;
                break;
            }
        }
    }
    if (!net->input_is_number) {
        for (c = 0; c < dims; c++)
            for (j = 0; j < N; j++) {
                if (j == net->ige) continue;
                input[c * N + j] *= net->unit[j];
                atol[c * N + j] *= net->unit[j];
            }
    }
    free(scale); free(prev); free(u0); free(s); free(gu); free(Ju);
    if (st) st->status = status;
    *dtp = dt;
    return ttot;
}

void dgo_evolve_cells(const dgo_network *net, const double *const *tables,
                      const double *dtf, double *dt, double z, double *input,
                      double *rtol, double *atol, long long ncells,
                      const dgo_config *cfg, double *ttot, int *status,
                      long long *substeps, long long *sweeps, long long *fails,
                      int nthreads)
{
    const int N = net->nchem;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        void *data = net->alloc_data(tables);
        long long c;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (c = 0; c < ncells; c++) {
            dgo_stats st;
            memset(&st, 0, sizeof(st));
            double d = dt[c];
            double t = dgo_evolve(net, data, dtf[c], &d, z, input + c * N, rtol + c * N,
                                  atol + c * N, 1, cfg, &st);
            dt[c] = d;
            if (ttot) ttot[c] = t;
            if (status) status[c] = st.status;
            if (substeps) substeps[c] = st.substeps_ok;
            if (sweeps) sweeps[c] = st.sweeps;
            if (fails) fails[c] = st.substeps_fail;
        }
        net->free_data(data);
    }
}

/* rates_and_rate_tables_run.pyx.template:124-178.  `input`, `atol`, `rtol`
 * are set by the caller (input = mass density / weight; atol = 1e-6*input;
 * rtol = 1e-6); electrons are made consistent here, after atol and the
 * scale were taken, as in the reference. */
int dgo_run_strip(const dgo_network *net, void *data, double tf, int niter,
                  double z, double *input, double *rtol, double *atol,
                  int dims, const dgo_config *cfg, double *ttot_out,
                  double *dt_out, dgo_stats *st)
{
    return dgo_run_strip_traj(net, data, tf, niter, z, input, rtol, atol, dims, cfg, ttot_out,
                              dt_out, st, NULL, NULL, NULL, NULL, NULL);
}

/* The same loop recording, per iteration taken, what the Cython driver's
 * intermediate arrays hold (run.pyx.template:146-175): the state after
 * BE_chem_solve (traj[(iter * dims + cell) * N + s]), the last temperature
 * computed (traj_T[iter * dims + cell]), the success flag, ttot and dt
 * before this iteration's update.  Each pointer may be NULL; entries of
 * iterations not taken are left as they are. */
int dgo_run_strip_traj(const dgo_network *net, void *data, double tf, int niter,
                       double z, double *input, double *rtol, double *atol,
                       int dims, const dgo_config *cfg, double *ttot_out,
                       double *dt_out, dgo_stats *st, double *traj, double *traj_T,
                       unsigned char *traj_ok, double *traj_t, double *traj_dt)
{
    const int N = net->nchem;
    const long long n = (long long)dims * N;
    long long i;
    int iter;
    double *prev = (double *)malloc(sizeof(double) * n);
    double *scale = (double *)malloc(sizeof(double) * n);
    double *u0 = (double *)malloc(sizeof(double) * n);
    double *s = (double *)malloc(sizeof(double) * N);
    double *gu = (double *)malloc(sizeof(double) * n);
    double *Ju = (double *)malloc(sizeof(double) * n * N);
    for (i = 0; i < n; i++) prev[i] = input[i];
    for (i = 0; i < n; i++) scale[i] = input[i];
    net->electrons(input, dims, N);
    net->set_z(data, z);
    double dt = tf / 1e5, ttot = 0.0;
    for (iter = 0; iter < niter; iter++) {
        int status = dgo_BE_chem_solve(net->rhs, net->jac, input, dt, rtol, atol, dims, N,
                                       scale, data, u0, s, gu, Ju, cfg->max_sweeps,
                                       st ? &st->sweeps : NULL);
        if (traj)
            for (i = 0; i < n; i++) traj[(long long)iter * n + i] = input[i];
        if (traj_T) {
            const double *Ts = net->Ts(data);
            for (i = 0; i < dims; i++) traj_T[(long long)iter * dims + i] = Ts[i];
        }
        if (traj_ok) traj_ok[iter] = status == 0 ? 1 : 0;
        if (traj_t) traj_t[iter] = ttot;
        if (traj_dt) traj_dt[iter] = dt;
        if (status == 0) {
            if (st) st->substeps_ok++;
            for (i = 0; i < n; i++) prev[i] = input[i];
            for (i = 0; i < n; i++) scale[i] = input[i];
            ttot += dt;
            dt *= 1.1;
            if (tf - ttot < dt) dt = tf - ttot;
        } else {
            if (st) st->substeps_fail++;
            dt /= 2.0;
            for (i = 0; i < n; i++) input[i] = prev[i];
            for (i = 0; i < n; i++) scale[i] = input[i];
            if (dt < 1e-30 * tf) {
                if (st) st->status = 2;
                break;
            }
            continue;
        }
        if (ttot >= tf) break;
    }
    free(prev); free(scale); free(u0); free(s); free(gu); free(Ju);
    *ttot_out = ttot;
    *dt_out = dt;
    return iter < niter ? iter + 1 : niter;
}

/* dgo_run_strip_traj on a data object built from `tables` (freed on return). */
int dgo_run_strip_tables(const dgo_network *net, const double *const *tables, double tf,
                         int niter, double z, double *input, double *rtol, double *atol,
                         int dims, const dgo_config *cfg, double *ttot_out, double *dt_out,
                         dgo_stats *st, double *traj, double *traj_T, unsigned char *traj_ok,
                         double *traj_t, double *traj_dt)
{
    void *data = net->alloc_data(tables);
    int it = dgo_run_strip_traj(net, data, tf, niter, z, input, rtol, atol, dims, cfg, ttot_out,
                                dt_out, st, traj, traj_T, traj_ok, traj_t, traj_dt);
    net->free_data(data);
    return it;
}

/* log x correctly rounded to double: a quad-precision log rounded once to
 * double (x86-64: libquadmath's logq, as its long double has only 64 bits
 * and rounding its log to double would round twice; AArch64: long double is
 * quad).  Checked against a 200-bit log in tests/test_oracle_golden.py. */
#if defined(__x86_64__)
#include <quadmath.h>
double dgo_crlog(double x) { return (double)logq((__float128)x); }
#else
double dgo_crlog(double x) { return (double)logl(x); }
#endif
