/*
 * The GB300 backward-Euler Newton engine: one cell per lane, the whole
 * per-cell solve (temperature, table interpolation, RHS, Jacobian, scaled
 * I - dt J, partial-pivot LU, Newton update and convergence vote, substep
 * accept/reject and dt control) fused into one kernel pass.
 *
 * Semantics are those of the reference's generated driver called with one
 * cell per strip (dims = 1), i.e. per-cell dt control:
 *   BE_chem_solve / BE_Resid_Fun / BE_Resid_Jac / Gauss_Elim
 *       dengo/solvers/BE_chem_solve.C:79-382
 *   dengo_evolve_<name>
 *       dengo/templates/rates_and_rate_tables.C.template:149-274
 * including the in-place atol round trips, the fixed scaling vector, the
 * floor at 1e-25 after an accepted substep (prev keeps the unfloored state),
 * the 50000-substep cap (the last solved state is returned unaccepted) and
 * the dt/dtf < 1e-15 stop.  The FP64 build performs the reference's IEEE
 * operations in the reference's order (no FMA contraction); dg_log /
 * dg_ipow stand in for glibc's log / pow.
 *
 * Lanes are refilled: when a lane's cell finishes it takes the next cell
 * (static stride or an atomic work queue) while the other lanes of its warp
 * continue, so a warp's lanes stay busy on a mix of stiff and easy cells.
 */
#ifndef DG_ENGINE_CUH
#define DG_ENGINE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "dg_math.h"
#include "dg_slots.cuh"
#include "dg_mixed.cuh"
#include "dg_xf.h"
#include "dengo_gb300.h"

namespace dg {

/* ST_SUSPENDED: set aside by the sweep budget; finished by a resume launch */
enum : int { ST_OK = 0, ST_MAX_SUBSTEPS = 1, ST_DT_UNDERFLOW = 2, ST_SUSPENDED = 3 };

/* Most tables a network with redshift tables may have: their values at a
 * call's z travel inside the kernel parameter (zvals below). */
#define DG_MAX_TABLES 64

/* Rate/cooling tables on the device, bin-major: for bin b and table k the
 * pair (r_k[b], r_k[b+1] - r_k[b]).  The difference is the reference's own
 * subtraction (rates_and_rate_tables.C.template:406-408) done once.
 * Passed by value to every kernel, so a launch carries its own z and its own
 * redshift-table values: no device buffer is written between calls and no
 * call waits for an earlier one. */
struct TableSet {
    const double2 *pairs;   /* [nbins][NT] */
    int nbins;              /* table length - 1 */
    double lb, dbin, idbin; /* log(T_lo), bin width, 1/width (host-computed) */
    double Tlo, Thi;
    double z;               /* redshift of this call (only compton-like terms read it) */
    double zvals[DG_MAX_TABLES]; /* [k]: value of redshift table k at z (host-computed;
                                    unused for the other tables) */
};

/* Cell arrays: element (cell c, species s) at p[c*cs + s*ss]. */
struct CellIO {
    double *state;
    double *atol;
    const double *rtol;
    double rtol_scalar;
    const double *dtf;
    double dtf_scalar;
    double *dt;
    double *ttot;
    int *status;
    int *substeps, *sweeps, *failures;
    const int *order;       /* optional: the q-th cell taken is order[q] */
    long long cs, ss;
    long long ncells;
};

struct KernelCfg {
    int max_sweeps;
    int max_substeps;
    double dt_ratio_floor;
    double floor_value;
    /* stiff-cell redistribution: a cell that has taken sweep_budget sweeps
     * (> 0) writes its suspension record at its next substep boundary and
     * ends with ST_SUSPENDED; with resume set, cells start from their record
     * instead of the input.  rec: rec_len<N>() doubles per cell. */
    int sweep_budget;
    int resume;
    double *rec;
    /* resume launch: the number of suspended cells (device) and the SM
     * count; only as many CTAs as give every SM one CTA per 32 (or BLOCK)
     * of those cells keep running, so a few stiff cells share warps rather
     * than competing CTAs */
    const unsigned int *resume_count;
    int nsm;
    /* mixed precision: the FP64 conservation check of every converged cell
     * -- a relative drift of any invariant beyond cons_tol re-solves the
     * cell with FP64 linear solves; 0: no check */
    double cons_tol;
    /* mixed precision: build the Newton matrix in extended-range FP32
     * (DENGO_MIXED_XF) instead of from FP64 products */
    int jac_xf;
    /* FP64 resume launch: when at most wide_max cells were set aside the
     * wide engine (dg_wide.cuh, one cell per CTA, wide_max CTAs) resumes
     * them and this engine's launch returns at once; 0: this engine resumes
     * them */
    int wide_max;
};

/* Suspension record of a cell at a substep boundary: state y, prev, scale,
 * atol (all unscaled number densities), dt, ttot, accepted substeps, sweeps,
 * failed substeps, and whether the cell is being re-solved in FP64 --
 * everything the driver carries between substeps. */
template <int N>
__host__ __device__ constexpr int rec_len() { return 4 * N + 6; }

template <class Net, int BLOCK, bool MIXED = false>
struct Lane {
    static constexpr int N = Net::N;
    static constexpr int NT = Net::NT;
    /* shared-memory slot map, in doubles per thread; the mixed path adds
     * the FP32 factors (half a slot per entry) after the FP64 matrix */
    static constexpr int OFF_J = 0;
    static constexpr int OFF_JF = OFF_J + N * N;
    static constexpr int OFF_R = OFF_JF + (MIXED ? (N * N + 1) / 2 : 0);
    static constexpr int OFF_PREV = OFF_R + NT;
    static constexpr int OFF_SC = OFF_PREV + N;
    static constexpr int OFF_INV = OFF_SC + N;
    static constexpr int OFF_AT = OFF_INV + N;
    static constexpr int OFF_RT = OFF_AT + N;
    static constexpr int SLOTS = OFF_RT + N;
    static constexpr size_t smem_bytes() { return sizeof(double) * SLOTS * BLOCK; }
};

/* Linear interpolation in log T (rates_and_rate_tables.C.template:372-411),
 * values only: the solver never reads the T-derivatives. */
template <class Net, int BLOCK>
__device__ __forceinline__ void interpolate(const TableSet &ts, double logT, Slots<BLOCK> R)
{
    const int bin = (int)(ts.idbin * (logT - ts.lb));
    const int bc = bin <= 0 ? 0 : (bin >= ts.nbins ? ts.nbins - 1 : bin);
    const double t1 = (ts.lb + (bin) * ts.dbin);
    const double t2 = (ts.lb + (bin + 1) * ts.dbin);
    const double Tdef = (logT - t1) / (t2 - t1);
    const double2 *row = ts.pairs + (size_t)bc * Net::NT;
#pragma unroll
    for (int k = 0; k < Net::NT; k++) {
        if (Net::zdep(k)) {
            R[k] = ts.zvals[k];
        } else {
            const double2 pr = __ldg(row + k);
            R[k] = pr.x + Tdef * pr.y;
        }
    }
}

/* Gauss_Elim (BE_chem_solve.C:330-382) on the scaled Jacobian held in
 * shared memory, column-major A(i,j) = J[j*N + i]; x holds b on entry and
 * the solution on exit. */
template <int N, int BLOCK>
__device__ __forceinline__ void gauss_elim(Slots<BLOCK> J, double (&x)[N])
{
#pragma unroll
    for (int k = 0; k < N - 1; k++) {
        int p = k;
        double best = fabs(J[k * N + k]);
#pragma unroll
        for (int i = k + 1; i < N; i++) {
            const double a = fabs(J[k * N + i]);
            if (a > best) {
                best = a;
                p = i;
            }
        }
        if (p != k) {
            for (int j = k; j < N; j++) {
                const double t = J[j * N + k];
                J[j * N + k] = J[j * N + p];
                J[j * N + p] = t;
            }
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                if (i == p) {
                    const double t = x[k];
                    x[k] = x[i];
                    x[i] = t;
                }
            }
        }
        const double piv = J[k * N + k];
#pragma unroll
        for (int i = k + 1; i < N; i++) J[k * N + i] = J[k * N + i] / piv;
#pragma unroll
        for (int j = k + 1; j < N; j++) {
            const double akj = J[j * N + k];
#pragma unroll
            for (int i = k + 1; i < N; i++) J[j * N + i] = J[j * N + i] - J[k * N + i] * akj;
        }
        const double xk = x[k];
#pragma unroll
        for (int i = k + 1; i < N; i++) x[i] = x[i] - J[k * N + i] * xk;
    }
#pragma unroll
    for (int i = N - 1; i >= 0; i--) {
        double xi = x[i];
#pragma unroll
        for (int j = i + 1; j < N; j++) xi = xi - J[j * N + i] * x[j];
        x[i] = xi / J[i * N + i];
    }
}

/* Gauss_Elim with the same result, fewer FP64 operations.
 *
 * Every entry the reference changes is computed with the reference's
 * operations in the reference's order, except that
 *   - a quotient by the pivot is formed as dg_div(a, piv, 1/piv), which is
 *     the correctly rounded a/piv, i.e. the reference's division;
 *   - an update a - m*b is skipped when m or b is an exact zero and the other
 *     factor is finite: then m*b is a zero and a - (+-0) == a (only the sign
 *     of an exactly-zero entry can differ, which no later comparison or
 *     nonzero result depends on).
 * The finiteness tests are per elimination step, so a row or multiplier set
 * holding inf/NaN is updated densely, exactly as the reference does. */
template <int N, int BLOCK>
__device__ __forceinline__ void gauss_elim_fast(Slots<BLOCK> J, double (&x)[N])
{
    double piv_v[N], piv_r[N];
#pragma unroll
    for (int k = 0; k < N - 1; k++) {
        int p = k;
        double best = J[k * N + k];
#pragma unroll
        for (int i = k + 1; i < N; i++) {
            const double a = J[k * N + i];
            if (dg_abs_gt(a, best)) {   /* fabs(a) > fabs(best) */
                best = a;
                p = i;
            }
        }
        if (p != k) {
            for (int j = k; j < N; j++) {
                const double t = J[j * N + k];
                J[j * N + k] = J[j * N + p];
                J[j * N + p] = t;
            }
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                if (i == p) {
                    const double t = x[k];
                    x[k] = x[i];
                    x[i] = t;
                }
            }
        }
        const double piv = J[k * N + k];
        const double rp = 1.0 / piv;
        piv_v[k] = piv;
        piv_r[k] = rp;
        double m[N], row[N];
        bool rowfin = true;
#pragma unroll
        for (int i = k + 1; i < N; i++) {
            m[i] = dg_div(J[k * N + i], piv, rp);
            J[k * N + i] = m[i];
        }
#pragma unroll
        for (int j = k + 1; j < N; j++) {
            row[j] = J[j * N + k];
            rowfin = rowfin && dg_finite(row[j]);
        }
#pragma unroll
        for (int i = k + 1; i < N; i++) {
            const bool mf = dg_finite(m[i]);
            if (dg_nonzero(m[i]) || !rowfin) {
#pragma unroll
                for (int j = k + 1; j < N; j++) {
                    if (dg_nonzero(row[j]) || !mf) J[j * N + i] = J[j * N + i] - m[i] * row[j];
                }
            }
        }
        const double xk = x[k];
        const bool xfin = dg_finite(xk);
#pragma unroll
        for (int i = k + 1; i < N; i++)
            if (dg_nonzero(m[i]) || !xfin) x[i] = x[i] - m[i] * xk;
    }
    piv_v[N - 1] = J[(N - 1) * N + (N - 1)];
    piv_r[N - 1] = 1.0 / piv_v[N - 1];
#pragma unroll
    for (int i = N - 1; i >= 0; i--) {
        double xi = x[i];
#pragma unroll
        for (int j = i + 1; j < N; j++) {
            const double aij = J[j * N + i];
            if (dg_nonzero(aij) || !dg_finite(x[j])) xi = xi - aij * x[j];
        }
        x[i] = dg_div(xi, piv_v[i], piv_r[i]);
    }
}

/* Stores one Jacobian entry already transformed as BE_Resid_Jac does:
 * row scale 1/scale_eq, column scale scale_var, then -dt*J, +1 on the
 * diagonal (BE_chem_solve.C:301-318).  zero() stores a structural zero:
 * when every scale is a positive finite number and dt > 0 the reference's
 * ((0 * inv) * scale) * -dt is -0.0 (1.0 on the diagonal), written directly;
 * otherwise (dense) the operations are carried out. */
template <int N, int BLOCK>
struct JacPut {
    Slots<BLOCK> J, INV, SC;
    double mdt;
    bool dense;
    __device__ __forceinline__ void operator()(int q, int v, double jv) const
    {
        double a = jv * INV[q];
        a = a * SC[v];
        a = mdt * a;
        if (q == v) a = a + 1.0;
        J[v * N + q] = a;
    }
    __device__ __forceinline__ void zero(int q, int v) const
    {
        if (dense) operator()(q, v, 0.0);
        else J[v * N + q] = (q == v) ? 1.0 : -0.0;
    }
};

/* The mixed-precision solve's Newton-matrix entry: BE_Resid_Jac's
 * ((J * inv_q) * scale_v) * -dt, + 1 on the diagonal (as JacPut), in
 * extended-range FP32 (dg_xf.h) -- each product rounded to FP32's 24-bit
 * significand, no FP64 instruction -- and stored as the (exact) FP64 value
 * of the result, which the equilibrated FP32 LU and the FP64 refinement
 * then use.  Only for cells whose scales are positive finite numbers and
 * dt > 0 (the FP64 Jacobian serves the others); zero() stores the
 * structural zero the reference computes there (-0.0, 1.0 on the
 * diagonal). */
template <int N, int BLOCK>
struct JacPutX {
    Slots<BLOCK> J, INV, SC;
    double mdt;
    __device__ __forceinline__ void operator()(int q, int v, XF jv) const
    {
        XF a = jv * xf(INV[q]);
        a = a * xf(SC[v]);
        a = a * xf(mdt);
        if (q == v) a = a + 1.0f;
        J[v * N + q] = xf_to_double(a);
    }
    __device__ __forceinline__ void zero(int q, int v) const
    {
        J[v * N + q] = (q == v) ? 1.0 : -0.0;
    }
};

/* Number-density conversion and electron consistency at the start of a
 * cell (rates_and_rate_tables.C.template:158-170). */
template <class Net>
__device__ __forceinline__ void to_number_density(double (&y)[Net::N], double (&at)[Net::N])
{
    if (!Net::INPUT_IS_NUMBER) {
#pragma unroll
        for (int s = 0; s < Net::N; s++) {
            if (s == Net::IGE) continue;
            y[s] = y[s] / Net::unit(s);
            at[s] = at[s] / Net::unit(s);
        }
    }
}

/* The FP64 conservation check of the mixed-precision solve: the invariants
 * of the network (Net::invariants, the species combinations its reactions
 * conserve) of a converged cell's final state y (number densities) against
 * those of its input, re-read from io.state and converted as at the cell's
 * start.  True when every relative drift |I(y) - I(y0)| / sum |c_s y0_s| is
 * within tol (a drift of exactly 0 always is).  The reference's own FP64
 * solve keeps these drifts near 1e-12 at most. */
template <class Net>
__device__ __forceinline__ bool conserved(const CellIO &io, long long cell,
                                          const double (&y)[Net::N], double tol)
{
    constexpr int N = Net::N;
    constexpr int NC = Net::NCONS > 0 ? Net::NCONS : 1;
    if (Net::NCONS == 0) return true;
    double y0[N], dummy[N];
#pragma unroll
    for (int s = 0; s < N; s++) {
        y0[s] = io.state[cell * io.cs + s * io.ss];
        dummy[s] = 0.0;
    }
    to_number_density<Net>(y0, dummy);
    Net::electrons(y0);
    double I0[NC], A0[NC], I1[NC], A1[NC];
    Net::invariants(y0, I0, A0);
    Net::invariants(y, I1, A1);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < Net::NCONS; k++) {
        const double d = fabs(I1[k] - I0[k]);
        ok = ok && !(d > tol * A0[k]);
    }
    return ok;
}

/* MIXED = false: the reference's FP64 arithmetic throughout (bit-faithful).
 * MIXED = true: the Newton matrix -- formed from FP64 products as the FP64
 * path forms it or, with cfg.jac_xf, built in extended-range FP32 (jacx,
 * JacPutX) -- is solved by MixedSolve (equilibrated FP32 LU + FP64
 * iterative refinement, dg_mixed.cuh), falling back to the FP64 Jacobian and
 * elimination for a cell whose matrix holds inf/NaN or whose scales are not
 * all positive and finite, and re-solving with FP64 linear solves a
 * converged cell that fails the FP64 conservation check; temperature,
 * rates, RHS, residual and the Newton update and its convergence test stay
 * FP64. */
template <class Net, int BLOCK, bool MIXED>
__global__ void __launch_bounds__(BLOCK)
evolve_kernel(CellIO io, TableSet ts, KernelCfg cfg, unsigned long long *queue)
{
    using L = Lane<Net, BLOCK, MIXED>;
    constexpr int N = Net::N;
    extern __shared__ double dg_smem[];
    const int tid = threadIdx.x;
    double *base = dg_smem + tid;
    const Slots<BLOCK> J{base + L::OFF_J * BLOCK};
    const SlotsF<BLOCK> JF{(float *)(dg_smem + L::OFF_JF * BLOCK) + tid};
    const Slots<BLOCK> R{base + L::OFF_R * BLOCK};
    const Slots<BLOCK> PREV{base + L::OFF_PREV * BLOCK};
    const Slots<BLOCK> SC{base + L::OFF_SC * BLOCK};
    const Slots<BLOCK> INV{base + L::OFF_INV * BLOCK};
    const Slots<BLOCK> AT{base + L::OFF_AT * BLOCK};
    const Slots<BLOCK> RT{base + L::OFF_RT * BLOCK};

    const long long stride = (long long)gridDim.x * BLOCK;
    if (cfg.resume && cfg.resume_count) {
        /* one lane per set-aside cell: a cell left waiting for a lane would
         * start its remaining ~10^5 sweeps only when another finished */
        const unsigned int cnt = *cfg.resume_count;
        if (cfg.wide_max > 0 && cnt <= (unsigned int)cfg.wide_max) return; /* wide engine's */
        const long long per_round = (long long)cfg.nsm * BLOCK;
        const long long rounds = ((long long)cnt + per_round - 1) / per_round;
        if (blockIdx.x >= cfg.nsm * (rounds > 0 ? rounds : 1)) return;
    }
    /* the work queue hands each warp 32 consecutive cells to start with (cells
     * adjacent in the order, alike in cost, share a warp) -- except when
     * resuming, where cells are spread over the CTAs; lanes then refill one
     * cell at a time */
    long long qi;
    {
        unsigned long long base = 0;
        const bool chunk = queue && !cfg.resume;
        if (chunk && (tid & 31) == 0) base = atomicAdd(queue, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        qi = chunk ? (long long)base + (tid & 31)
                   : (queue ? (long long)atomicAdd(queue, 1ull) : (long long)blockIdx.x * BLOCK + tid);
    }
    long long cell = 0;
    bool dense = false;   /* a scale is not a positive finite number */
    bool fp64cell = false;  /* mixed: this cell is re-solved with FP64 linear solves */

    double u[N], u0[N], y[N];
    double dtf = 0, dt = 0, ttot = 0;
    int siter = 0, isweep = 0, nsweeps = 0, nfail = 0;
    bool active = false;

    /* ---- helpers as lambdas over the lane's state ---- */
    auto substep_begin = [&]() {
        /* BE_chem_solve.C:93-117 */
#pragma unroll
        for (int i = 0; i < N; i++) u[i] = y[i] * INV[i];
#pragma unroll
        for (int i = 0; i < N; i++) AT[i] = AT[i] * INV[i];
#pragma unroll
        for (int i = 0; i < N; i++) u0[i] = u[i];
        isweep = 0;
    };
    /* from_record: continue a suspended cell (resume launch); else start it
     * from the caller's input */
    auto cell_begin = [&](bool from_record) -> bool {
        if (from_record) {
            /* continue a suspended cell from its record */
            const double *rc = cfg.rec + cell * rec_len<N>();
            dense = false;
#pragma unroll
            for (int s = 0; s < N; s++) {
                y[s] = rc[s];
                PREV[s] = rc[N + s];
                SC[s] = rc[2 * N + s];
                AT[s] = rc[3 * N + s];
                RT[s] = io.rtol ? io.rtol[cell * io.cs + s * io.ss] : io.rtol_scalar;
                INV[s] = 1.0 / SC[s];
                dense = dense || !(SC[s] > 0.0 && dg_finite(SC[s]));
            }
            dtf = io.dtf ? io.dtf[cell] : io.dtf_scalar;
            dt = rc[4 * N];
            ttot = rc[4 * N + 1];
            siter = (int)rc[4 * N + 2];
            nsweeps = (int)rc[4 * N + 3];
            nfail = (int)rc[4 * N + 4];
            fp64cell = rc[4 * N + 5] != 0.0;
            if (!(ttot < dtf)) return false;
            substep_begin();
            return true;
        }
        double at[N];
#pragma unroll
        for (int s = 0; s < N; s++) {
            const long long off = cell * io.cs + s * io.ss;
            y[s] = io.state[off];
            at[s] = io.atol[off];
            RT[s] = io.rtol ? io.rtol[off] : io.rtol_scalar;
        }
        to_number_density<Net>(y, at);
        Net::electrons(y);
#pragma unroll
        for (int s = 0; s < N; s++) AT[s] = at[s];
        dtf = io.dtf ? io.dtf[cell] : io.dtf_scalar;
        dt = io.dt ? io.dt[cell] : -1.0;
        if (dt < 0) dt = dtf / 1e5;
        ttot = 0;
        siter = 0;
        nsweeps = 0;
        nfail = 0;
        dense = false;
#pragma unroll
        for (int s = 0; s < N; s++) {
            SC[s] = y[s];
            PREV[s] = y[s];
            INV[s] = 1.0 / y[s];
            dense = dense || !(y[s] > 0.0 && dg_finite(y[s]));
        }
        if (!(ttot < dtf)) return false;
        substep_begin();
        return true;
    };
    auto cell_end = [&](int status) {
#pragma unroll
        for (int s = 0; s < N; s++) {
            double v = y[s], a = AT[s];
            if (!Net::INPUT_IS_NUMBER && s != Net::IGE) {
                v = v * Net::unit(s);
                a = a * Net::unit(s);
            }
            const long long off = cell * io.cs + s * io.ss;
            io.state[off] = v;
            io.atol[off] = a;
        }
        if (io.dt) io.dt[cell] = dt;
        if (io.ttot) io.ttot[cell] = ttot;
        if (io.status) io.status[cell] = status;
        if (io.substeps) io.substeps[cell] = siter;
        if (io.sweeps) io.sweeps[cell] = nsweeps;
        if (io.failures) io.failures[cell] = nfail;
    };
    auto suspend = [&]() {
        double *rc = cfg.rec + cell * rec_len<N>();
#pragma unroll
        for (int s = 0; s < N; s++) {
            rc[s] = y[s];
            rc[N + s] = PREV[s];
            rc[2 * N + s] = SC[s];
            rc[3 * N + s] = AT[s];
        }
        rc[4 * N] = dt;
        rc[4 * N + 1] = ttot;
        rc[4 * N + 2] = siter;
        rc[4 * N + 3] = nsweeps;
        rc[4 * N + 4] = nfail;
        rc[4 * N + 5] = fp64cell ? 1.0 : 0.0;
        io.status[cell] = ST_SUSPENDED;
    };
    auto fetch = [&]() {
        while (qi < io.ncells) {
            cell = io.order ? (long long)io.order[qi] : qi;
            if (cell < 0) break; /* end of a resume list */
            fp64cell = false;
            if (cell_begin(cfg.resume != 0)) {
                active = true;
                return;
            }
            cell_end(ST_OK);
            qi = queue ? (long long)atomicAdd(queue, 1ull) : qi + stride;
        }
        active = false;
    };

    fetch();
    while (active) {
        /* ---------------- one Newton sweep ---------------- */
        bool ok, unsolved = false, nan = false;
        double T, Tge;
        {
            /* BE_Resid_Fun (BE_chem_solve.C:246-275) */
#pragma unroll
            for (int i = 0; i < N; i++) y[i] = u[i] * SC[i];
            Net::temperature(y, ts.Tlo, ts.Thi, T, Tge);
            interpolate<Net, BLOCK>(ts, dg_log(T), R);
            double f[N];
            ok = Net::rhs(y, R, T, ts.z, f);
            if (ok) {
#pragma unroll
                for (int i = 0; i < N; i++) u[i] = y[i] * INV[i];
#pragma unroll
                for (int i = 0; i < N; i++) f[i] = f[i] * INV[i];
#pragma unroll
                for (int i = 0; i < N; i++) f[i] = u[i] - u0[i] - dt * f[i];
                /* BE_Resid_Jac (BE_chem_solve.C:280-321) */
#pragma unroll
                for (int i = 0; i < N; i++) y[i] = u[i] * SC[i];
                const bool dense_j = dense || !(dt > 0.0);
                if (MIXED && cfg.jac_xf && !dense_j && !fp64cell) {
                    /* the Jacobian in extended-range FP32 */
                    const JacPutX<N, BLOCK> put{J, INV, SC, -dt};
                    ok = Net::jacx(y, R, Tge, T, ts.z, put);
                } else {
                    const JacPut<N, BLOCK> put{J, INV, SC, -dt, dense_j};
                    ok = Net::jac(y, R, Tge, T, ts.z, put);
                }
                if (ok) {
#pragma unroll
                    for (int i = 0; i < N; i++) u[i] = y[i] * INV[i];
                    bool solved = false;
                    if (MIXED && !dense_j && !fp64cell) {
                        double xs[N];
                        solved = MixedSolve<Net, BLOCK>{J, JF}(f, xs);
                        if (solved) {
#pragma unroll
                            for (int i = 0; i < N; i++) f[i] = xs[i];
                        }
                    }
                    if (!solved) gauss_elim_fast<N, BLOCK>(J, f);
                    /* Newton update and max-norm test (BE_chem_solve.C:173-206) */
#pragma unroll
                    for (int i = 0; i < N; i++) u[i] = u[i] - 1.0 * f[i];
#pragma unroll
                    for (int i = 0; i < N; i++) {
                        /* fabs(s) > atol + rtol*fabs(u), then the NaN test */
                        if (dg_abs_gt_val(f[i], AT[i] + RT[i] * fabs(u[i]))) {
                            unsolved = true;
                            break;
                        }
                        if (dg_isnan(u[i])) {
                            nan = true;
                            break;
                        }
                    }
                }
            }
        }
        isweep++;
        nsweeps++;
        int rv = -1;
        if (!ok || nan) rv = 1;
        else if (!unsolved) rv = 0;
        else if (isweep >= cfg.max_sweeps) rv = 1;
        if (rv < 0) continue;

        /* ---------- end of BE_chem_solve: unscale (BE_chem_solve.C:225-239) ---------- */
#pragma unroll
        for (int i = 0; i < N; i++) y[i] = u[i] * SC[i];
#pragma unroll
        for (int i = 0; i < N; i++) AT[i] = AT[i] * SC[i];
        /* ---------- substep accept / reject (C.template:197-255) ---------- */
        if (rv == 0) {
#pragma unroll
            for (int i = 0; i < N; i++)
                if (dg_lt0(y[i])) rv = 1;
        }
        int done = -1;
        if (rv == 0) {
            if (siter == cfg.max_substeps) {
                done = ST_MAX_SUBSTEPS;
            } else {
                siter++;
                ttot += dt;
                const double grown = dt * 1.1, rest = dtf - ttot;
                dt = grown < rest ? grown : rest;
#pragma unroll
                for (int i = 0; i < N; i++) {
                    PREV[i] = y[i];
                    if (dg_lt_pos(y[i], cfg.floor_value)) y[i] = cfg.floor_value;
                }
                if (!(ttot < dtf)) done = ST_OK;
            }
        } else {
            nfail++;
            dt /= 2.0;
#pragma unroll
            for (int i = 0; i < N; i++) y[i] = PREV[i];
            if (dt / dtf < cfg.dt_ratio_floor) done = ST_DT_UNDERFLOW;
        }
        if (done < 0 && !(cfg.sweep_budget > 0 && nsweeps >= cfg.sweep_budget)) {
            substep_begin();
            continue;
        }
        if (MIXED && done == ST_OK && cfg.cons_tol != 0.0 && !fp64cell &&
            !conserved<Net>(io, cell, y, cfg.cons_tol)) {
            /* start the cell again from its input, FP64 linear solves */
            fp64cell = true;
            if (cell_begin(false)) continue;
        }
        if (done < 0) suspend();
        else cell_end(done);
        qi = queue ? (long long)atomicAdd(queue, 1ull) : qi + stride;
        fetch();
    }
}

}  // namespace dg
#endif
