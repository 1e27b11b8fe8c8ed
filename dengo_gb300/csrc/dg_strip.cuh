/*
 * Kernels behind the reference's strip-wise entry points, one thread per
 * cell of a strip (AoS input, input[cell*nchem + species]):
 *   <n>_calculate_temperature  rates_and_rate_tables.C.template:309-350
 *   <n>_interpolate_rates      rates_and_rate_tables.C.template:362-455
 *   calculate_rhs_<n>          rates_and_rate_tables.C.template:460-522
 *   calculate_jacobian_<n>     rates_and_rate_tables.C.template:527-599
 *   ensure_electron_consistency  rates_and_rate_tables.C.template:604-630
 *   temperature_from_mass_density  rates_and_rate_tables.C.template:635-668
 * Per-strip quantities live in device arrays laid out like the reference's
 * data struct fields: Ts[cell], rs[table][cell], ...
 */
#ifndef DG_STRIP_CUH
#define DG_STRIP_CUH

#include "dg_engine.cuh"

namespace dg {

struct StripBufs {
    double *Ts, *logTs, *invTs, *dTs_ge, *Tdef, *dT;
    double *rs, *drs;   /* [NT][ld] */
    int *bin_id;
    int *flag;          /* per cell: 1 if a species was negative */
    long long ld;       /* leading dimension of rs/drs */
};

/* Column accessor over a [table][cell] array. */
struct ColumnRates {
    const double *p;
    long long ld;
    __device__ __forceinline__ double operator[](int k) const { return p[k * ld]; }
};

template <class Net>
__device__ __forceinline__ void load_cell(const double *in, int nchem, int c, double (&y)[Net::N])
{
#pragma unroll
    for (int s = 0; s < Net::N; s++) y[s] = in[(long long)c * nchem + s];
}

/* Table interpolation into a per-thread array (values only). */
template <class Net>
__device__ __forceinline__ void interpolate_local(const TableSet &ts, double logT, double *R)
{
    const int bin = (int)(ts.idbin * (logT - ts.lb));
    const int bc = bin <= 0 ? 0 : (bin >= ts.nbins ? ts.nbins - 1 : bin);
    const double t1 = (ts.lb + (bin) * ts.dbin);
    const double t2 = (ts.lb + (bin + 1) * ts.dbin);
    const double Tdef = (logT - t1) / (t2 - t1);
    const double2 *row = ts.pairs + (size_t)bc * Net::NT;
    for (int k = 0; k < Net::NT; k++) {
        if (Net::zdep(k)) {
            R[k] = ts.zvals[k];
        } else {
            const double2 pr = row[k];
            R[k] = pr.x + Tdef * pr.y;
        }
    }
}

template <class Net>
__global__ void strip_temperature_kernel(const double *in, int nstrip, int nchem, TableSet ts,
                                         StripBufs b)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nstrip) return;
    double y[Net::N];
    load_cell<Net>(in, nchem, c, y);
    double T, Tge;
    Net::temperature(y, ts.Tlo, ts.Thi, T, Tge);
    b.Ts[c] = T;
    b.logTs[c] = dg_log(T);
    b.invTs[c] = 1.0 / T;
    b.dTs_ge[c] = Tge;
}

/* zv/dzv: values and z-derivatives of the redshift tables at this call's z
 * (host-computed; zero when z is outside the tabulated range). */
template <class Net>
__global__ void strip_interpolate_kernel(int nstrip, TableSet ts, StripBufs b, const double *zv,
                                         const double *dzv)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nstrip) return;
    const double logT = b.logTs[c];
    const int bin = (int)(ts.idbin * (logT - ts.lb));
    const int bc = bin <= 0 ? 0 : (bin >= ts.nbins ? ts.nbins - 1 : bin);
    const double t1 = (ts.lb + (bin) * ts.dbin);
    const double t2 = (ts.lb + (bin + 1) * ts.dbin);
    const double Tdef = (logT - t1) / (t2 - t1);
    const double dT = (t2 - t1);
    b.bin_id[c] = bc;
    b.Tdef[c] = Tdef;
    b.dT[c] = dT;
    const double invT = b.invTs[c];
    const double2 *row = ts.pairs + (size_t)bc * Net::NT;
    for (int k = 0; k < Net::NT; k++) {
        double v, dv;
        if (Net::zdep(k)) {
            v = zv[k];
            dv = dzv[k];
        } else {
            const double2 pr = row[k];
            v = pr.x + Tdef * pr.y;
            dv = pr.y;
            dv = dv / dT;
            dv = dv * invT;
        }
        b.rs[k * b.ld + c] = v;
        b.drs[k * b.ld + c] = dv;
    }
}

template <class Net>
__global__ void strip_rhs_kernel(const double *in, double *out, int nstrip, int nchem,
                                 double z, StripBufs b)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nstrip) return;
    double y[Net::N], f[Net::N];
    load_cell<Net>(in, nchem, c, y);
    const ColumnRates R{b.rs + c, b.ld};
    const bool ok = Net::rhs(y, R, b.Ts[c], z, f);
    b.flag[c] = ok ? 0 : 1;
    if (!ok) return;
#pragma unroll
    for (int s = 0; s < Net::N; s++) out[(long long)c * nchem + s] = f[s];
}

struct PlainPut {
    double *J;
    int N;
    __device__ __forceinline__ void operator()(int q, int v, double jv) const { J[v * N + q] = jv; }
    __device__ __forceinline__ void zero(int q, int v) const { J[v * N + q] = 0.0; }
};

template <class Net>
__global__ void strip_jacobian_kernel(const double *in, double *J, int nstrip, int nchem,
                                      double z, StripBufs b)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nstrip) return;
    double y[Net::N];
    load_cell<Net>(in, nchem, c, y);
    const ColumnRates R{b.rs + c, b.ld};
    const PlainPut put{J + (long long)c * Net::N * Net::N, Net::N};
    const bool ok = Net::jac(y, R, b.dTs_ge[c], b.Ts[c], z, put);
    b.flag[c] = ok ? 0 : 1;
}

/* The reference accumulates total_e across the whole strip without
 * resetting it per cell; reproduced by one thread walking the cells. */
template <class Net>
__global__ void strip_electrons_kernel(double *in, int nstrip, int nchem)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double total_e = 0.0;
    for (int c = 0; c < nstrip; c++) {
        double y[Net::N];
        load_cell<Net>(in, nchem, c, y);
        total_e = Net::electron_sum(y, total_e);
        if (Net::IDE >= 0) in[(long long)c * nchem + Net::IDE] = total_e;
    }
}

template <class Net>
__global__ void strip_temperature_from_mass_kernel(const double *in, int nstrip, int nchem,
                                                   double *T)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nstrip) return;
    double y[Net::N];
    load_cell<Net>(in, nchem, c, y);
    T[c] = Net::temperature_from_mass_density(y);
}

/* Longest-first cell order from a per-cell cost hint (e.g. the sweeps the
 * cell needed in the previous hydro step): 32 buckets by floor(log2(cost+1)),
 * costliest bucket first; the order inside a bucket is arbitrary (results do
 * not depend on it).  counts/offsets hold 32 ints each, zeroed by the caller. */
__device__ __forceinline__ int cost_bucket(int c)
{
    const unsigned v = (unsigned)(c < 0 ? 0 : c) + 1u;
    return __clz(v);   /* 31 - floor(log2 v): big costs get small buckets */
}

static __global__ void order_count_kernel(const int *cost, long long n, int *counts)
{
    __shared__ int sc[32];
    if (threadIdx.x < 32) sc[threadIdx.x] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        atomicAdd(&sc[cost_bucket(cost[i])], 1);
    __syncthreads();
    if (threadIdx.x < 32 && sc[threadIdx.x]) atomicAdd(&counts[threadIdx.x], sc[threadIdx.x]);
}

static __global__ void order_scan_kernel(const int *counts, int *offsets)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int run = 0;
    for (int b = 0; b < 32; b++) {
        offsets[b] = run;
        run += counts[b];
    }
}

static __global__ void order_scatter_kernel(const int *cost, long long n, int *offsets, int *order)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        order[atomicAdd(&offsets[cost_bucket(cost[i])], 1)] = (int)i;
}

/* The resume list of a redistributed solve (sweep budget): list[0..count) = the suspended
 * cells (any order), then -1 (the end marker the engines stop at). */
static __global__ void resume_list_fill_kernel(int *list, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        list[i] = -1;
}

static __global__ void resume_list_kernel(const int *status, long long n, int *list,
                                          unsigned int *count)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        if (status[i] == ST_SUSPENDED) list[atomicAdd(count, 1u)] = (int)i;
}

/* Scaled Jacobian store into a per-thread array (BE_chem_solve.C:301-318). */
template <int N>
struct ScaledLocalPut {
    double *J;
    const double *inv, *sc;
    double mdt;
    __device__ __forceinline__ void operator()(int q, int v, double jv) const
    {
        double a = jv * inv[q];
        a = a * sc[v];
        a = mdt * a;
        if (q == v) a = a + 1.0;
        J[v * N + q] = a;
    }
    __device__ __forceinline__ void zero(int q, int v) const { operator()(q, v, 0.0); }
};

template <int N>
__device__ void gauss_elim_local(double *A, double *x)
{
    for (int k = 0; k < N - 1; k++) {
        int p = k;
        for (int i = k + 1; i < N; i++)
            if (fabs(A[k * N + i]) > fabs(A[k * N + p])) p = i;
        for (int j = k; j < N; j++) {
            const double t = A[j * N + k];
            A[j * N + k] = A[j * N + p];
            A[j * N + p] = t;
        }
        const double t = x[k];
        x[k] = x[p];
        x[p] = t;
        for (int i = k + 1; i < N; i++) A[k * N + i] /= A[k * N + k];
        for (int j = k + 1; j < N; j++)
            for (int i = k + 1; i < N; i++) A[j * N + i] -= A[k * N + i] * A[j * N + k];
        for (int i = k + 1; i < N; i++) x[i] -= A[k * N + i] * x[k];
    }
    for (int i = N - 1; i >= 0; i--) {
        for (int j = i + 1; j < N; j++) x[i] -= A[j * N + i] * x[j];
        x[i] /= A[i * N + i];
    }
}

/* BE_chem_solve (BE_chem_solve.C:79-241) over one strip in lockstep, on the
 * per-thread state of a block with one thread per cell (act: the thread has
 * a cell; c: its index).  All cells share the sweep loop; a negative value
 * anywhere fails the strip at the RHS or Jacobian stage, a NaN stops the
 * sweep at the first such cell in cell order (later cells keep their
 * pre-update values), and the strip converges only when every cell passed
 * the max-norm test.  u and at are updated as the reference writes them back
 * (unscaled); T receives the cell's last temperature.  Returns the
 * reference's return value, the same in every thread.  first_bad: one int
 * of shared memory.  Every thread of the block must call it. */
template <class Net>
__device__ int be_strip_solve(bool act, int c, int nstrip, double (&u)[Net::N], double (&at)[Net::N],
                              const double (&rt)[Net::N], const double (&sc)[Net::N], double dt,
                              const TableSet &ts, int max_sweeps, double &T, int *first_bad)
{
    constexpr int N = Net::N;
    double us[N], u0[N], inv[N], y[N], g[N], upre[N];
    double R[Net::NT];
    double A[N * N];
    if (act) {
        for (int i = 0; i < N; i++) {
            inv[i] = 1.0 / sc[i];
            us[i] = u[i] * inv[i];
            at[i] = at[i] * inv[i];
            u0[i] = us[i];
        }
    }
    int rv = 1;
    int fail_mode = 0; /* 0 none, 1 u = y*sc (RHS/Jacobian failure) */
    for (int isweep = 0; isweep < max_sweeps; isweep++) {
        bool ok = true;
        double Tge = 0;
        if (act) {
            for (int i = 0; i < N; i++) y[i] = us[i] * sc[i];
            Net::temperature(y, ts.Tlo, ts.Thi, T, Tge);
            interpolate_local<Net>(ts, dg_log(T), R);
            ok = Net::rhs(y, R, T, ts.z, g);
        }
        if (__syncthreads_or(act && !ok)) {
            fail_mode = 1;
            break;
        }
        if (act) {
            for (int i = 0; i < N; i++) us[i] = y[i] * inv[i];
            for (int i = 0; i < N; i++) g[i] = g[i] * inv[i];
            for (int i = 0; i < N; i++) g[i] = us[i] - u0[i] - dt * g[i];
            for (int i = 0; i < N; i++) y[i] = us[i] * sc[i];
            const ScaledLocalPut<N> put{A, inv, sc, -dt};
            ok = Net::jac(y, R, Tge, T, ts.z, put);
        }
        if (__syncthreads_or(act && !ok)) {
            fail_mode = 1;
            break;
        }
        bool unsolved = false, nan = false;
        if (act) {
            for (int i = 0; i < N; i++) us[i] = y[i] * inv[i];
            gauss_elim_local<N>(A, g);
            for (int i = 0; i < N; i++) upre[i] = us[i];
            for (int i = 0; i < N; i++) us[i] -= 1.0 * g[i];
            for (int i = 0; i < N; i++) {
                if (fabs(g[i]) > (at[i] + rt[i] * fabs(us[i]))) {
                    unsolved = true;
                    break;
                }
                if (us[i] != us[i]) {
                    nan = true;
                    break;
                }
            }
        }
        if (c == 0) *first_bad = nstrip;
        __syncthreads();
        if (act && nan) atomicMin(first_bad, c);
        __syncthreads();
        const int fb = *first_bad;
        __syncthreads();
        if (fb < nstrip) {
            if (act && c > fb)
                for (int i = 0; i < N; i++) us[i] = upre[i];
            rv = 1;
            break;
        }
        const bool any_unsolved = __syncthreads_or(act && unsolved);
        rv = any_unsolved ? 1 : 0;
        if (!any_unsolved) break;
    }
    if (act) {
        for (int i = 0; i < N; i++) {
            u[i] = fail_mode ? y[i] * sc[i] : us[i] * sc[i];
            at[i] = at[i] * sc[i];
        }
    }
    return fail_mode ? 1 : rv;
}

/* BE_chem_solve as a kernel: one block, one thread per cell; u, atol
 * (number densities, AoS) updated in place, the return value in *ret and
 * each cell's last temperature in Ts. */
template <class Net>
__global__ void __launch_bounds__(DENGO_MAX_NCELLS)
be_strip_kernel(double *u, double dt, const double *rtol, double *atol, int nstrip,
                const double *scaling, TableSet ts, int max_sweeps, int *ret, double *Ts)
{
    constexpr int N = Net::N;
    const int c = threadIdx.x;
    const bool act = c < nstrip;
    __shared__ int first_bad;
    double us[N], sc[N], at[N], rt[N];
    if (act) {
        for (int i = 0; i < N; i++) {
            sc[i] = scaling[c * N + i];
            us[i] = u[c * N + i];
            at[i] = atol[c * N + i];
            rt[i] = rtol[c * N + i];
        }
    }
    double T = 0;
    const int rv = be_strip_solve<Net>(act, c, nstrip, us, at, rt, sc, dt, ts, max_sweeps, T,
                                       &first_bad);
    if (act) {
        for (int i = 0; i < N; i++) {
            u[c * N + i] = us[i];
            atol[c * N + i] = at[i];
        }
        Ts[c] = T;
    }
    if (c == 0) *ret = rv;
}

/* Per-strip control state of a lockstep evolve (evolve_lockstep_kernel),
 * kept in device memory so that a launch can stop after an accepted substep
 * and the next launch resume. */
struct LockStrip {
    double dt, ttot;
    int siter;
    int status;   /* 0 running or integrated to dtf, 1 substep cap, 2 dt floor */
    int done;     /* the strip's evolve has ended */
    int dumped;   /* this launch ended at an accepted substep (dump written) */
};

/* Arguments of evolve_lockstep_kernel.  input/atol/rtol: the caller's AoS
 * arrays (mass densities + ge unless the network takes number densities),
 * cells [b*strip, min(dims, (b+1)*strip)) form strip b.  rec: per cell
 * rec_len<N>() doubles (u, prev, scale, atol in number densities, then T)
 * for a launch that stops after an accepted substep; dump: per cell N + 1
 * doubles (prev and T at that substep). */
struct LockIO {
    double *input, *atol;
    const double *rtol;
    long long dims;
    int strip;
    double dtf;
    LockStrip *ls;
    double *rec, *dump;
    int resume, stop_after_accept;
};

/* dengo_evolve_<n> (rates_and_rate_tables.C.template:149-274) over strips
 * in lockstep, the reference's semantics for dims > 1: one CTA per strip,
 * one thread per cell; mass -> number densities (input and atol), the
 * electron consistency with the reference's running total over the strip,
 * dt = dtf / 1e5 when the caller's dt < 0, scale = prev = input fixed for the
 * call; then while ttot < dtf: BE_chem_solve over the whole strip (one dt,
 * one Newton loop), any negative value anywhere fails the substep; on
 * success: stop at the substep cap, siter++, ttot += dt,
 * dt = min(1.1 dt, dtf - ttot), [intermediate dump of prev and T], prev =
 * input, values below floor_value raised to it; on failure: dt /= 2,
 * input = prev, stop when dt / dtf < dt_ratio_floor; finally number -> mass
 * densities.  With stop_after_accept the launch returns after each accepted
 * substep (its state in rec) so that the host can write the reference's
 * <n>_intermediate_%06d file (C.template:212-241) before resuming. */
template <class Net>
__global__ void __launch_bounds__(DENGO_MAX_NCELLS)
evolve_lockstep_kernel(LockIO io, TableSet ts, KernelCfg cfg)
{
    constexpr int N = Net::N;
    constexpr int RL = rec_len<N>();
    const long long first = (long long)blockIdx.x * io.strip;
    const long long left = io.dims - first;
    const int nstrip = (int)(left < io.strip ? left : io.strip);
    const int c = threadIdx.x;
    const bool act = c < nstrip;
    const long long cell = first + c;
    LockStrip &L = io.ls[blockIdx.x];
    __shared__ int first_bad;
    if (L.done) return;
    double u[N], prev[N], sc[N], at[N], rt[N];
    double T = 0;
    double dt, ttot;
    int siter;
    if (!io.resume) {
        if (act) {
            for (int i = 0; i < N; i++) {
                u[i] = io.input[cell * N + i];
                at[i] = io.atol[cell * N + i];
                rt[i] = io.rtol[cell * N + i];
            }
            to_number_density<Net>(u, at);
            for (int i = 0; i < N; i++) io.input[cell * N + i] = u[i];
        }
        __syncthreads();
        if (c == 0) {
            /* ensure_electron_consistency: the running total over the strip */
            double total = 0.0;
            for (int k = 0; k < nstrip; k++) {
                double y[N];
                for (int i = 0; i < N; i++) y[i] = io.input[(first + k) * N + i];
                total = Net::electron_sum(y, total);
                if (Net::IDE >= 0) io.input[(first + k) * N + Net::IDE] = total;
            }
        }
        __syncthreads();
        if (act)
            for (int i = 0; i < N; i++) {
                u[i] = io.input[cell * N + i];
                sc[i] = u[i];
                prev[i] = u[i];
            }
        dt = L.dt < 0 ? io.dtf / 1e5 : L.dt;
        ttot = 0.0;
        siter = 0;
    } else {
        if (act) {
            const double *r = io.rec + cell * RL;
            for (int i = 0; i < N; i++) {
                u[i] = r[i];
                prev[i] = r[N + i];
                sc[i] = r[2 * N + i];
                at[i] = r[3 * N + i];
                rt[i] = io.rtol[cell * N + i];
            }
        }
        dt = L.dt;
        ttot = L.ttot;
        siter = L.siter;
    }
    /* every thread has read the strip record before thread 0 may write it */
    __syncthreads();
    int status = 0;
    bool stopped = false;
    while (ttot < io.dtf) {
        int rv = be_strip_solve<Net>(act, c, nstrip, u, at, rt, sc, dt, ts, cfg.max_sweeps, T,
                                     &first_bad);
        bool neg = false;
        if (act)
            for (int i = 0; i < N; i++) neg = neg || dg_lt0(u[i]);
        if (__syncthreads_or(neg)) rv = 1;
        if (rv == 0) {
            if (siter == cfg.max_substeps) {
                status = 1;
                break;
            }
            siter++;
            ttot += dt;
            const double grown = dt * 1.1, rest = io.dtf - ttot;
            dt = grown < rest ? grown : rest;
            if (io.stop_after_accept && act) {
                double *dp = io.dump + cell * (N + 1);
                for (int i = 0; i < N; i++) dp[i] = prev[i];
                dp[N] = T;
            }
            if (act)
                for (int i = 0; i < N; i++) {
                    prev[i] = u[i];
                    if (dg_lt_pos(u[i], cfg.floor_value)) u[i] = cfg.floor_value;
                }
            if (io.stop_after_accept && ttot < io.dtf) {
                stopped = true;
                break;
            }
        } else {
            dt /= 2.0;
            if (act)
                for (int i = 0; i < N; i++) u[i] = prev[i];
            if (dt / io.dtf < cfg.dt_ratio_floor) {
                status = 2;
                break;
            }
        }
    }
    if (stopped) {
        if (act) {
            double *r = io.rec + cell * RL;
            for (int i = 0; i < N; i++) {
                r[i] = u[i];
                r[N + i] = prev[i];
                r[2 * N + i] = sc[i];
                r[3 * N + i] = at[i];
            }
        }
        if (c == 0) {
            L.dt = dt;
            L.ttot = ttot;
            L.siter = siter;
            L.dumped = 1;
        }
        return;
    }
    if (act) {
        if (!Net::INPUT_IS_NUMBER) {
            for (int i = 0; i < N; i++) {
                if (i == Net::IGE) continue;
                u[i] = u[i] * Net::unit(i);
                at[i] = at[i] * Net::unit(i);
            }
        }
        for (int i = 0; i < N; i++) {
            io.input[cell * N + i] = u[i];
            io.atol[cell * N + i] = at[i];
        }
    }
    if (c == 0) {
        /* an evolve that ended right after an accepted substep still hands
         * that substep's dump to the host */
        L.dumped = io.stop_after_accept && status == 0 && siter > 0 && !(ttot < io.dtf) ? 1 : 0;
        L.dt = dt;
        L.ttot = ttot;
        L.siter = siter;
        L.status = status;
        L.done = 1;
    }
}

/* Outputs of run_strip_kernel; the trajectory arrays may be null. */
struct RunOut {
    double *ttot, *dt;   /* [1] */
    int *iters;          /* [1]: iterations taken (the reference's iter + 1) */
    double *traj;        /* [niter][nstrip][N] state after each BE_chem_solve */
    double *traj_T;      /* [niter][nstrip] last temperature of each solve */
    unsigned char *traj_ok; /* [niter] 1 when the solve converged */
    double *traj_t, *traj_dt; /* [niter] ttot and dt at each solve */
};

/* The Cython driver run_<n> (rates_and_rate_tables_run.pyx.template:114-205)
 * on one strip in lockstep, after its mass-to-number conversion: prev and
 * scale start as the input, the electrons are made consistent (the
 * reference's running total over the strip), dt = tf/1e5; then up to niter
 * BE_chem_solve calls: on success prev = scale = u, ttot += dt, dt *= 1.1,
 * dt clipped to tf - ttot, stop when ttot >= tf; on failure dt /= 2,
 * u = scale = prev, stop when dt < 1e-30 tf. */
template <class Net>
__global__ void __launch_bounds__(DENGO_MAX_NCELLS)
run_strip_kernel(double *input, const double *rtol, double *atol, int nstrip, double tf, int niter,
                 TableSet ts, int max_sweeps, RunOut out)
{
    constexpr int N = Net::N;
    const int c = threadIdx.x;
    const bool act = c < nstrip;
    __shared__ int first_bad;
    double u[N], prev[N], sc[N], at[N], rt[N];
    if (act) {
        for (int i = 0; i < N; i++) {
            prev[i] = input[c * N + i];
            sc[i] = prev[i];
            at[i] = atol[c * N + i];
            rt[i] = rtol[c * N + i];
        }
    }
    __syncthreads();
    if (c == 0) {
        /* ensure_electron_consistency over the strip, in cell order */
        double total = 0.0;
        for (int k = 0; k < nstrip; k++) {
            double y[N];
            for (int i = 0; i < N; i++) y[i] = input[k * N + i];
            total = Net::electron_sum(y, total);
            if (Net::IDE >= 0) input[k * N + Net::IDE] = total;
        }
    }
    __syncthreads();
    if (act)
        for (int i = 0; i < N; i++) u[i] = input[c * N + i];
    double dt = tf / 1e5, ttot = 0.0;
    int iter = 0;
    for (; iter < niter; iter++) {
        double T = 0;
        const int status = be_strip_solve<Net>(act, c, nstrip, u, at, rt, sc, dt, ts, max_sweeps,
                                               T, &first_bad);
        if (out.traj && act)
            for (int i = 0; i < N; i++) out.traj[((size_t)iter * nstrip + c) * N + i] = u[i];
        if (out.traj_T && act) out.traj_T[(size_t)iter * nstrip + c] = T;
        if (c == 0) {
            if (out.traj_ok) out.traj_ok[iter] = status == 0;
            if (out.traj_t) out.traj_t[iter] = ttot;
            if (out.traj_dt) out.traj_dt[iter] = dt;
        }
        if (status == 0) {
            if (act)
                for (int i = 0; i < N; i++) {
                    prev[i] = u[i];
                    sc[i] = u[i];
                }
            ttot += dt;
            dt *= 1.1;
            if (tf - ttot < dt) dt = tf - ttot;
        } else {
            dt /= 2.0;
            if (act)
                for (int i = 0; i < N; i++) {
                    u[i] = prev[i];
                    sc[i] = u[i];
                }
            if (dt < 1e-30 * tf) break;
            continue;
        }
        if (ttot >= tf) break;
    }
    if (act)
        for (int i = 0; i < N; i++) {
            input[c * N + i] = u[i];
            atol[c * N + i] = at[i];
        }
    if (c == 0) {
        *out.ttot = ttot;
        *out.dt = dt;
        *out.iters = iter < niter ? iter + 1 : niter;
    }
}

}  // namespace dg
#endif
