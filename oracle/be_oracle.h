/*
 * ORACLE -- test infrastructure, not part of the product.
 *
 * A plain-C restatement of the reference's backward-Euler Newton solver and
 * its time-step driver, used only as the checker: by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  Nothing in
 * dengo_gb300/ links or calls it.
 *
 * Reference:
 *   BE_chem_solve / BE_Resid_Fun / BE_Resid_Jac / Gauss_Elim
 *       dengo/solvers/BE_chem_solve.C:79-382
 *   dengo_evolve_<name>
 *       dengo/templates/rates_and_rate_tables.C.template:149-274
 *   run_<name> (Cython driver)
 *       dengo/templates/rates_and_rate_tables_run.pyx.template:81-205
 *
 * Built with -O2 -ffp-contract=off (no FMA contraction) so that it performs
 * the same IEEE operations as the reference compiled on x86-64.
 */
#ifndef DGO_BE_ORACLE_H
#define DGO_BE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int (*dgo_rhs_f)(double *, double *, int, int, void *);
typedef int (*dgo_jac_f)(double *, double *, int, int, void *);

/* One network's generated functions (oracle/gen/<name>_oracle.c). */
typedef struct {
    const char *name;
    int nchem;
    int ige;
    const double *unit;     /* weight * 1.67e-24 per species (unused for ge) */
    int input_is_number;
    dgo_rhs_f rhs;
    dgo_jac_f jac;
    void (*electrons)(double *input, int nstrip, int nchem);
    void *(*alloc_data)(const double *const *tables);
    void (*free_data)(void *);
    void (*set_z)(void *data, double z);
    const double *(*Ts)(const void *data);
} dgo_network;

/* Solver constants; dgo_default_config() returns the reference's values. */
typedef struct {
    int max_sweeps;          /* BE_chem_solve.C:87                 */
    int max_substeps;        /* C.template:204                     */
    double dt_ratio_floor;   /* C.template:251  (dt/dtf < 1e-15)   */
    double floor_value;      /* C.template:187                     */
} dgo_config;

/* Per-call counters (summed over the cells of the call). */
typedef struct {
    long long substeps_ok;    /* accepted substeps                 */
    long long substeps_fail;  /* rejected substeps (dt halved)     */
    long long sweeps;         /* Newton sweeps (RHS+J+LU each)     */
    int status;               /* 0 ok, 1 substep cap, 2 dt underflow */
} dgo_stats;

dgo_config dgo_default_config(void);

int dgo_BE_chem_solve(dgo_rhs_f f, dgo_jac_f J, double *u, double dt,
                      double *rtol, double *atol, int nstrip, int nchem,
                      double *scaling, void *sdata, double *u0, double *s,
                      double *gu, double *Ju, int max_sweeps, long long *sweeps);

int dgo_Gauss_Elim(double *A, double *x, double *b, int n);

double dgo_evolve(const dgo_network *net, void *data, double dtf, double *dt,
                  double z, double *input, double *rtol, double *atol,
                  long long dims, const dgo_config *cfg, dgo_stats *st);

/* Called by dgo_evolve where the reference writes <name>_intermediate_%06d
 * (rates_and_rate_tables.C.template:212-241), with what it writes: the
 * accepted substep's number, prev (the state before that substep, number
 * densities, dims x N), the data's Ts, ttot and the next dt.  NULL: off. */
typedef void (*dgo_intermediate_f)(void *ctx, int siter, const double *prev,
                                   const double *Ts, long long dims, int nchem,
                                   double ttot, double dt);
void dgo_set_intermediate_hook(dgo_intermediate_f f, void *ctx);

/* Per-cell driver: every cell is its own strip (dims = 1), the reference's
 * dengo_evolve called once per cell.  AoS in/out like the reference.
 * dt[c] < 0 selects dtf[c]/1e5.  Runs cells on `nthreads` OpenMP threads. */
void dgo_evolve_cells(const dgo_network *net, const double *const *tables,
                      const double *dtf, double *dt, double z, double *input,
                      double *rtol, double *atol, long long ncells,
                      const dgo_config *cfg, double *ttot, int *status,
                      long long *substeps, long long *sweeps, long long *fails,
                      int nthreads);

/* The Cython driver run_<name> (run.pyx.template:114-205) for one strip,
 * starting from number densities already divided by the weights.
 * Returns the number of loop iterations executed. */
int dgo_run_strip(const dgo_network *net, void *data, double tf, int niter,
                  double z, double *input, double *rtol, double *atol,
                  int dims, const dgo_config *cfg, double *ttot_out,
                  double *dt_out, dgo_stats *st);

/* dgo_run_strip recording the Cython driver's intermediate arrays
 * (run.pyx.template:146-175); each trajectory pointer may be NULL. */
int dgo_run_strip_traj(const dgo_network *net, void *data, double tf, int niter,
                       double z, double *input, double *rtol, double *atol,
                       int dims, const dgo_config *cfg, double *ttot_out,
                       double *dt_out, dgo_stats *st, double *traj, double *traj_T,
                       unsigned char *traj_ok, double *traj_t, double *traj_dt);

/* dgo_run_strip_traj on a data object built from the tables (freed on
 * return). */
int dgo_run_strip_tables(const dgo_network *net, const double *const *tables, double tf,
                         int niter, double z, double *input, double *rtol, double *atol,
                         int dims, const dgo_config *cfg, double *ttot_out, double *dt_out,
                         dgo_stats *st, double *traj, double *traj_T, unsigned char *traj_ok,
                         double *traj_t, double *traj_dt);

/* log x correctly rounded (long double log rounded to double) */
double dgo_crlog(double x);

#ifdef __cplusplus
}
#endif
#endif
