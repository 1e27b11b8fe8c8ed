/*
 * Split engine: 32 cells per CTA, one per lane, and the Newton sweep of each
 * cell divided over NP cooperating warps (NP = 2 or 4), which the scheduler
 * places on different SM sub-partitions and hence different FP64 units.
 *
 * On GB300 each sub-partition's FP64 unit accepts one warp instruction every
 * ~64 cycles whatever the number of active lanes, so a cell's sweep costs
 * about (FP64 instructions on its path) x 64 cycles.  The stiffest cells need
 * 10^5 sequential sweeps and set the length of a hydro step; splitting a sweep
 * over NP warps shortens that path by up to NP while each FP64 warp
 * instruction still serves 32 cells.
 *
 * Work split of one sweep (barriers between phases):
 *   warp 0        substep bookkeeping; the convergence decision; cell refill
 *                 (work queue)
 *   warp 1 % NP   T(ge), log T, bin
 *   warp 2 % NP   pivot search and row swap (FP64 elimination); mixed: the
 *                 FP32 factorisation and first solve
 *   warp 3 % NP   back substitution (FP64 elimination); mixed: the
 *                 refinement's FP32 corrections
 *   all warps     table interpolation (tables k = w mod NP), RHS rows and
 *                 Jacobian entries of part w (generated partition balanced by
 *                 operation count); for rows i = w mod NP: the residual, the
 *                 LU multipliers and row updates, the Newton update and the
 *                 row's max-norm / NaN test (mixed: the refinement residual)
 * Every value is computed with exactly the operations of the single-lane
 * engine (dg_engine.cuh), so results are bit-identical to it and hence to the
 * reference.  Per-cell state lives in shared memory as [slot][32] doubles.
 */
#ifndef DG_SPLIT_CUH
#define DG_SPLIT_CUH

#include "dg_engine.cuh"

namespace dg {

template <class Net, int NP, bool MIXED>
struct SplitLayout {
    static constexpr int N = Net::N;
    static constexpr int NT = Net::NT;
    static constexpr int J = 0;           /* FP64 matrix */
    /* The rates are dead once the Jacobian is built, so the mixed path's
     * FP32 factors and refined solution share their region. */
    static constexpr int R = J + N * N;   /* rates */
    static constexpr int JF = R;          /* mixed: FP32 factors */
    static constexpr int X = JF + (N * N + 1) / 2;   /* mixed: refined solution */
    static constexpr int RSZ = MIXED ? (NT > X + N - R ? NT : X + N - R) : NT;
    static constexpr int Y = R + RSZ;     /* unscaled state seen by RHS/Jacobian */
    static constexpr int G = Y + N;       /* RHS, residual, Newton update */
    static constexpr int U = G + N;
    static constexpr int U0 = U + N;
    static constexpr int SC = U0 + N;
    static constexpr int INV = SC + N;
    static constexpr int AT = INV + N;
    static constexpr int RT = AT + N;
    static constexpr int PREV = RT + N;
    static constexpr int SCAL = PREV + N;  /* T, Tge, Tdef, -dt, piv, 1/piv */
    static constexpr int RPV = SCAL + 6;    /* FP64 path: 1/pivot of each step */
    static constexpr int SLOTS = RPV + (MIXED ? 0 : N);
    static constexpr int NFLAGS = 10 + N;  /* 10 cell flags, then one per row (F_ROW + i) */
    /* per-cell ints after the doubles: NFLAGS flags, then (mixed) the row
     * and column scale exponents and the FP32 pivots, N each */
    static constexpr int NINTS = NFLAGS + (MIXED ? 3 * N : 0);
    static constexpr size_t bytes() { return sizeof(double) * SLOTS * 32 + sizeof(int) * NINTS * 32 + 64; }
};

/* per-cell int flags; F_MIX: 0 FP64 elimination, 1 refining, 2 refined;
 * F_FP64: mixed precision, the cell is re-solved with FP64 linear solves
 * (it failed the conservation check) */
enum : int { F_ACT = 0, F_BIN = 1, F_OKR = 2, F_OKJ = 3, F_DENSE = 4, F_PIV = 5, F_SWEEP = 6,
             F_MIX = 7, F_EPREV = 8, F_FP64 = 9, F_ROW = 10 };

/* The FP64 elimination for a cell the mixed solve hands back (dense or
 * non-finite system); kept out of line because it is rarely taken and large. */
template <int N>
__device__ __noinline__ void fp64_fallback(Slots<32> J, Slots<32> G)
{
    double g[N];
    for (int i = 0; i < N; i++) g[i] = G[i];
    gauss_elim_fast<N, 32>(J, g);
    for (int i = 0; i < N; i++) G[i] = g[i];
}

/* The mixed variant is held to the register budget of three 4-warp CTAs per
 * SM, the occupancy its shared memory allows for the 10-species network. */
template <class Net, int NP, bool MIXED>
__global__ void __launch_bounds__(32 * NP, MIXED ? 3 : 1)
evolve_split_kernel(CellIO io, TableSet ts, KernelCfg cfg, unsigned long long *queue)
{
    using L = SplitLayout<Net, NP, MIXED>;
    constexpr int N = Net::N;
    extern __shared__ double dg_smem[];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    /* The per-cell serial phases go to different warps, so that with
     * several CTAs per SM they need not all queue on one sub-partition's
     * FP64 unit: the control (warp 0), T(ge) and log T (W_T), the pivot
     * search or the mixed path's FP32 factorisation (W_PIV), the back
     * substitution or the refinement's corrections (W_BS).  (On the
     * config-2 bench's first step, three CTAs per SM, the time did not
     * change measurably: 15.37 s before, 15.46 s after.) */
    constexpr int W_T = 1 % NP, W_PIV = 2 % NP, W_BS = 3 % NP;
    double *cellbase = dg_smem + l;
    const Slots<32> J{cellbase + L::J * 32}, R{cellbase + L::R * 32}, Y{cellbase + L::Y * 32},
        G{cellbase + L::G * 32}, U{cellbase + L::U * 32}, U0{cellbase + L::U0 * 32},
        SC{cellbase + L::SC * 32}, INV{cellbase + L::INV * 32}, AT{cellbase + L::AT * 32},
        RT{cellbase + L::RT * 32}, PREV{cellbase + L::PREV * 32}, S{cellbase + L::SCAL * 32},
        RPV{cellbase + L::RPV * 32};
    const SlotsF<32> JF{(float *)(dg_smem + L::JF * 32) + l};
    int *iflags = (int *)(dg_smem + L::SLOTS * 32);
    auto F = [&](int f) -> int & { return iflags[f * 32 + l]; };
    /* mixed: s (row exponents), t (column exponents), FP32 pivots */
    auto MI = [&](int k) -> int & { return iflags[(L::NFLAGS + k) * 32 + l]; };
    const Slots<32> X{cellbase + L::X * 32};
    __shared__ int s_any;

    /* warp-0 control state of this lane's cell */
    long long qi = 0, cell = 0;
    double dtf = 0, dt = 0, ttot = 0;
    int siter = 0, isweep = 0, nsweeps = 0, nfail = 0;
    bool active = false, dense = false;
    const long long stride = (long long)gridDim.x * 32;
    if (cfg.resume && cfg.resume_count) {
        /* one lane per set-aside cell: a cell left waiting for a lane would
         * start its remaining ~10^5 sweeps only when another finished */
        const unsigned int cnt = *cfg.resume_count;
        if (cfg.wide_max > 0 && cnt <= (unsigned int)cfg.wide_max) return; /* wide engine's */
        const long long per_round = (long long)cfg.nsm * 32;
        const long long rounds = ((long long)cnt + per_round - 1) / per_round;
        if (blockIdx.x >= cfg.nsm * (rounds > 0 ? rounds : 1)) return;
    }
    if (w == 0) {
        /* the work queue hands each CTA 32 consecutive cells to start with, so
         * cells adjacent in the order (alike in cost) share a CTA -- except
         * when resuming, where cells are spread over the CTAs; lanes then
         * refill one cell at a time */
        unsigned long long base = 0;
        const bool chunk = queue && !cfg.resume;
        if (chunk && l == 0) base = atomicAdd(queue, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        qi = chunk ? (long long)base + l
                   : (queue ? (long long)atomicAdd(queue, 1ull) : (long long)blockIdx.x * 32 + l);
    }

    auto substep_begin = [&]() {
        for (int i = 0; i < N; i++) {
            const double v = Y[i] * INV[i];
            U[i] = v;
            U0[i] = v;
            AT[i] = AT[i] * INV[i];
        }
        isweep = 0;
    };
    /* from_record: continue a suspended cell (resume launch); else start it
     * from the caller's input */
    auto cell_begin = [&](bool from_record) -> bool {
        if (from_record) {
            /* continue a suspended cell from its record */
            const double *rc = cfg.rec + cell * rec_len<N>();
            dense = false;
            for (int s = 0; s < N; s++) {
                Y[s] = rc[s];
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
            F(F_FP64) = rc[4 * N + 5] != 0.0;
            if (!(ttot < dtf)) return false;
            substep_begin();
            return true;
        }
        double y[N], at[N];
        for (int s = 0; s < N; s++) {
            const long long off = cell * io.cs + s * io.ss;
            y[s] = io.state[off];
            at[s] = io.atol[off];
            RT[s] = io.rtol ? io.rtol[off] : io.rtol_scalar;
        }
        to_number_density<Net>(y, at);
        Net::electrons(y);
        dtf = io.dtf ? io.dtf[cell] : io.dtf_scalar;
        dt = io.dt ? io.dt[cell] : -1.0;
        if (dt < 0) dt = dtf / 1e5;
        ttot = 0;
        siter = nsweeps = nfail = 0;
        dense = false;
        for (int s = 0; s < N; s++) {
            AT[s] = at[s];
            Y[s] = y[s];
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
        for (int s = 0; s < N; s++) {
            double v = Y[s], a = AT[s];
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
        for (int s = 0; s < N; s++) {
            rc[s] = Y[s];
            rc[N + s] = PREV[s];
            rc[2 * N + s] = SC[s];
            rc[3 * N + s] = AT[s];
        }
        rc[4 * N] = dt;
        rc[4 * N + 1] = ttot;
        rc[4 * N + 2] = siter;
        rc[4 * N + 3] = nsweeps;
        rc[4 * N + 4] = nfail;
        rc[4 * N + 5] = F(F_FP64) ? 1.0 : 0.0;
        io.status[cell] = ST_SUSPENDED;
    };
    auto fetch = [&]() {
        while (qi < io.ncells) {
            cell = io.order ? (long long)io.order[qi] : qi;
            if (cell < 0) break; /* end of a resume list */
            F(F_FP64) = 0;
            if (cell_begin(cfg.resume != 0)) {
                active = true;
                return;
            }
            cell_end(ST_OK);
            qi = queue ? (long long)atomicAdd(queue, 1ull) : qi + stride;
        }
        active = false;
    };

    if (w == 0) {
        fetch();
        F(F_ACT) = active;
    }
    __syncthreads();   /* the first cells' state, read by warp W_T */
    for (;;) {
        /* ---- P0: the control warp publishes -dt; warp W_T unscales the
         *      state and forms T(ge), log T and the bin ---- */
        if (w == 0) {
            const unsigned anyact = __ballot_sync(0xffffffffu, active);
            if (l == 0) s_any = anyact != 0;
            if (active) {
                S[3] = -dt;
                F(F_DENSE) = dense || !(dt > 0.0);
            }
            F(F_OKR) = 1;
            F(F_OKJ) = 1;
        }
        if (w == W_T && F(F_ACT)) {
            double y[N];
            for (int i = 0; i < N; i++) {
                y[i] = U[i] * SC[i];
                Y[i] = y[i];
            }
            double T, Tge;
            Net::temperature(y, ts.Tlo, ts.Thi, T, Tge);
            const double logT = dg_log(T);
            const int bin = (int)(ts.idbin * (logT - ts.lb));
            const int bc = bin <= 0 ? 0 : (bin >= ts.nbins ? ts.nbins - 1 : bin);
            const double t1 = (ts.lb + (bin) * ts.dbin);
            const double t2 = (ts.lb + (bin + 1) * ts.dbin);
            S[0] = T;
            S[1] = Tge;
            S[2] = (logT - t1) / (t2 - t1);
            F(F_BIN) = bc;
        }
        __syncthreads();
        if (!s_any) break;
        const bool act = F(F_ACT) != 0;
        /* ---- P1 (all warps): interpolation, tables k = w mod NP ---- */
        if (act) {
            const double Tdef = S[2];
            const double2 *row = ts.pairs + (size_t)F(F_BIN) * Net::NT;
            for (int k = w; k < Net::NT; k += NP) {
                if (Net::zdep(k)) {
                    R[k] = ts.zvals[k];
                } else {
                    const double2 pr = __ldg(row + k);
                    R[k] = pr.x + Tdef * pr.y;
                }
            }
        }
        __syncthreads();
        /* ---- P2 (all warps): RHS rows of part w ---- */
        if (act) {
            double y[N], f[N];
            for (int i = 0; i < N; i++) y[i] = Y[i];
            bool ok = true;
            switch (w) {
            case 0: ok = Net::template rhs<NP, 0>(y, R, S[0], ts.z, f); break;
            case 1: ok = Net::template rhs<NP, 1 % NP>(y, R, S[0], ts.z, f); break;
            case 2: ok = Net::template rhs<NP, 2 % NP>(y, R, S[0], ts.z, f); break;
            default: ok = Net::template rhs<NP, 3 % NP>(y, R, S[0], ts.z, f); break;
            }
            if (ok) {
                for (int i = 0; i < N; i++)
                    if (Net::rhs_row_part(NP, i) == w) G[i] = f[i];
            } else {
                atomicAnd(&F(F_OKR), 0);
            }
        }
        __syncthreads();
        /* ---- P3 (all warps, rows i = w mod NP): residual g = u - u0 - dt f
         *      (scaled), y for the Jacobian ---- */
        if (act && F(F_OKR)) {
            const double dtv = -S[3];
            for (int i = w; i < N; i += NP) {
                const double u = Y[i] * INV[i];
                double g = G[i] * INV[i];
                g = u - U0[i] - dtv * g;
                G[i] = g;
                U[i] = u;
                Y[i] = u * SC[i];
                if (MIXED) MI(N + i) = MixedSolve<Net, 32>::NONE;
            }
        }
        __syncthreads();
        /* ---- P4 (all warps): Jacobian entries of part w, scaled ---- */
        const bool do_j = act && F(F_OKR);
        if (do_j) {
            double y[N];
            for (int i = 0; i < N; i++) y[i] = Y[i];
            bool ok = true;
            if (MIXED && cfg.jac_xf && !F(F_DENSE) && !F(F_FP64)) {
                /* mixed: the Jacobian in extended-range FP32 */
                const JacPutX<N, 32> put{J, INV, SC, S[3]};
                switch (w) {
                case 0: ok = Net::template jacx<NP, 0>(y, R, S[1], S[0], ts.z, put); break;
                case 1: ok = Net::template jacx<NP, 1 % NP>(y, R, S[1], S[0], ts.z, put); break;
                case 2: ok = Net::template jacx<NP, 2 % NP>(y, R, S[1], S[0], ts.z, put); break;
                default: ok = Net::template jacx<NP, 3 % NP>(y, R, S[1], S[0], ts.z, put); break;
                }
            } else {
                const JacPut<N, 32> put{J, INV, SC, S[3], F(F_DENSE) != 0};
                switch (w) {
                case 0: ok = Net::template jac<NP, 0>(y, R, S[1], S[0], ts.z, put); break;
                case 1: ok = Net::template jac<NP, 1 % NP>(y, R, S[1], S[0], ts.z, put); break;
                case 2: ok = Net::template jac<NP, 2 % NP>(y, R, S[1], S[0], ts.z, put); break;
                default: ok = Net::template jac<NP, 3 % NP>(y, R, S[1], S[0], ts.z, put); break;
                }
            }
            if (!ok) atomicAnd(&F(F_OKJ), 0);
        }
        __syncthreads();
        const bool do_lu = do_j && F(F_OKJ);
        /* u = y / scale after the Jacobian (rows i = w mod NP; the mixed
         * refinement below reuses Y for the residual of the same rows) */
        if (do_lu)
            for (int i = w; i < N; i += NP) U[i] = Y[i] * INV[i];
        /* ---- P5: LU.  FP64: pivot (warp 0) then row updates (all warps).
         *      Mixed: equilibrated FP32 factorisation and first solve on
         *      warp 0; each refinement's FP64 residual rows i = w mod NP on
         *      all warps, the FP32 correction on warp 0; the single-lane FP64
         *      elimination for a dense or non-finite system ---- */
        if (MIXED) {
            using MS = MixedSolve<Net, 32>;
            const MS ms{J, JF};
            const bool eq = do_lu && !F(F_DENSE) && !F(F_FP64);
            /* M1 (rows i = w mod NP): row scale exponent s_i, finiteness of
             * the row and of g_i, and the row's share of each column's
             * largest scaled exponent (MI(N + j), reset to NONE in P3) */
            if (eq) {
#pragma unroll
                for (int i = 0; i < N; i++) {
                    if (i % NP != w) continue;
                    int m = 0;
                    bool fin = dg_expo(G[i]) != 0x7ff;
#pragma unroll
                    for (int j = 0; j < N; j++) {
                        const int e = dg_expo(J[j * N + i]);
                        fin = fin && e != 0x7ff;
                        m = e > m ? e : m;
                    }
                    const int si = m ? 1022 - m : 0;
                    MI(i) = si;
                    F(F_ROW + i) = fin;
#pragma unroll
                    for (int j = 0; j < N; j++) {
                        if (!Net::jnz(i, j)) continue;
                        const int e = dg_expo(J[j * N + i]);
                        if (e != 0) atomicMax(&MI(N + j), e + si);
                    }
                }
            }
            __syncthreads();
            /* M2 (rows i = w mod NP): R A C rounded to FP32 */
            if (eq) {
#pragma unroll
                for (int i = 0; i < N; i++) {
                    if (i % NP != w) continue;
                    const int si = MI(i);
#pragma unroll
                    for (int j = 0; j < N; j++) {
                        const int cm = MI(N + j);
                        const int tj = cm == MS::NONE ? 0 : 1022 - cm;
                        JF[j * N + i] = Net::jnz(i, j) ? dg_f32_scaled(J[j * N + i], si + tj) : 0.0f;
                    }
                }
            }
            __syncthreads();
            /* M3 (warp W_PIV): FP32 factorisation and first solve; the
             * FP64 elimination for a dense or non-finite system */
            if (w == W_PIV && do_lu) {
                double g[N], x[N];
                int sx[N], tx[N], px[N];
                bool ok = eq;
                for (int i = 0; i < N; i++) {
                    g[i] = G[i];
                    ok = ok && F(F_ROW + i);
                }
                if (ok) {
                    for (int i = 0; i < N; i++) {
                        sx[i] = MI(i);
                        const int cm = MI(N + i);
                        tx[i] = cm == MS::NONE ? 0 : 1022 - cm;
                    }
                    ms.factor(px);
                    int ed;
                    ok = ms.apply(px, sx, tx, g, x, ed);
                }
                if (ok) {
                    for (int i = 0; i < N; i++) {
                        MI(N + i) = tx[i];
                        MI(2 * N + i) = px[i];
                        X[i] = x[i];
                    }
                    F(F_MIX) = 1;
                    F(F_EPREV) = 0x7ff;
                } else {
                    fp64_fallback<N>(J, G);
                    F(F_MIX) = 0;
                }
            }
            __syncthreads();
            for (int it = 0; it < MixedSolve<Net, 32>::MAX_REFINE; it++) {
                const bool refining = do_lu && F(F_MIX) == 1;
                if (!__syncthreads_or(refining)) break;
                if (refining) {
#pragma unroll
                    for (int i = 0; i < N; i++)
                        if (i % NP == w) Y[i] = ms.residual_row(i, G[i], X);
                }
                __syncthreads();
                if (w == W_BS && refining) {
                    double r[N], x[N];
                    int sx[N], tx[N], px[N];
                    for (int i = 0; i < N; i++) {
                        r[i] = Y[i];
                        x[i] = X[i];
                        sx[i] = MI(i);
                        tx[i] = MI(N + i);
                        px[i] = MI(2 * N + i);
                    }
                    int eprev = F(F_EPREV);
                    bool more;
                    if (ms.refine(px, sx, tx, r, x, eprev, more)) {
                        for (int i = 0; i < N; i++) X[i] = x[i];
                        F(F_EPREV) = eprev;
                        F(F_MIX) = more ? 1 : 2;
                        if (DG_MIXED_STRICT && !more && !MS::refined(x, eprev)) F(F_MIX) = 3;
                    } else {
                        fp64_fallback<N>(J, G);
                        F(F_MIX) = 0;
                    }
                }
                __syncthreads();
            }
#if DG_MIXED_STRICT
            /* refinement stopped short of 2^-40 (3) or ran out of steps (1) */
            if (w == W_BS && do_lu && (F(F_MIX) == 1 || F(F_MIX) == 3)) {
                fp64_fallback<N>(J, G);
                F(F_MIX) = 0;
            }
#endif
            if (w == W_BS && do_lu && F(F_MIX) != 0)
                for (int i = 0; i < N; i++) G[i] = X[i];
        } else {
            for (int k = 0; k < N - 1; k++) {
                __syncthreads();
                if (w == W_PIV && do_lu) {
                    int p = k;
                    double best = J[k * N + k];
                    for (int i = k + 1; i < N; i++) {
                        const double a = J[k * N + i];
                        if (dg_abs_gt(a, best)) {
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
                        const double t = G[k];
                        G[k] = G[p];
                        G[p] = t;
                    }
                    const double piv = J[k * N + k];
                    const double rp = 1.0 / piv;
                    S[4] = piv;
                    S[5] = rp;
                    RPV[k] = rp;   /* reused by the back substitution */
                }
                __syncthreads();
                if (do_lu) {
                    const double piv = S[4], rp = S[5];
                    bool rowfin = true;
                    for (int j = k + 1; j < N; j++) rowfin = rowfin && dg_finite(J[j * N + k]);
                    const double xk = G[k];
                    const bool xfin = dg_finite(xk);
                    for (int i = k + 1 + ((w - (k + 1) % NP + NP) % NP); i < N; i += NP) {
                        const double m = dg_div(J[k * N + i], piv, rp);
                        J[k * N + i] = m;
                        const bool mf = dg_finite(m);
                        if (dg_nonzero(m) || !rowfin) {
                            for (int j = k + 1; j < N; j++) {
                                const double akj = J[j * N + k];
                                if (dg_nonzero(akj) || !mf) J[j * N + i] = J[j * N + i] - m * akj;
                            }
                        }
                        if (dg_nonzero(m) || !xfin) G[i] = G[i] - m * xk;
                    }
                }
            }
            __syncthreads();
            if (w == W_BS && do_lu) {
                /* back substitution; the pivots are the final diagonal and
                 * their reciprocals were formed during the elimination */
                RPV[N - 1] = 1.0 / J[(N - 1) * N + (N - 1)];
                for (int i = N - 1; i >= 0; i--) {
                    double xi = G[i];
                    for (int j = i + 1; j < N; j++) {
                        const double aij = J[j * N + i];
                        const double xj = G[j];
                        if (dg_nonzero(aij) || !dg_finite(xj)) xi = xi - aij * xj;
                    }
                    G[i] = dg_div(xi, J[i * N + i], RPV[i]);
                }
            }
        }
        __syncthreads();
        /* ---- P6a (all warps, rows i = w mod NP): Newton update and each
         *      row's max-norm / NaN test ---- */
        if (act && F(F_OKR) && F(F_OKJ)) {
            for (int i = w; i < N; i += NP) {
                const double u = U[i] - 1.0 * G[i];
                U[i] = u;
                F(F_ROW + i) = dg_abs_gt_val(G[i], AT[i] + RT[i] * fabs(u)) ? 1 : (dg_isnan(u) ? 2 : 0);
            }
        }
        __syncthreads();
        /* ---- P6b (warp 0): the first row that fails decides, as in the
         *      reference's row loop; substep control ---- */
        if (w == 0 && act) {
            bool ok = F(F_OKR) && F(F_OKJ), unsolved = false, nan = false;
            if (ok) {
                for (int i = 0; i < N; i++) {
                    const int r = F(F_ROW + i);
                    if (r) {
                        unsolved = r == 1;
                        nan = r == 2;
                        break;
                    }
                }
            }
            isweep++;
            nsweeps++;
            int rv = -1;
            if (!ok || nan) rv = 1;
            else if (!unsolved) rv = 0;
            else if (isweep >= cfg.max_sweeps) rv = 1;
            if (rv >= 0) {
                double y[N];
                for (int i = 0; i < N; i++) {
                    y[i] = U[i] * SC[i];
                    AT[i] = AT[i] * SC[i];
                }
                if (rv == 0)
                    for (int i = 0; i < N; i++)
                        if (dg_lt0(y[i])) rv = 1;
                int done = -1;
                if (rv == 0) {
                    if (siter == cfg.max_substeps) {
                        done = ST_MAX_SUBSTEPS;
                    } else {
                        siter++;
                        ttot += dt;
                        const double grown = dt * 1.1, rest = dtf - ttot;
                        dt = grown < rest ? grown : rest;
                        for (int i = 0; i < N; i++) {
                            PREV[i] = y[i];
                            if (dg_lt_pos(y[i], cfg.floor_value)) y[i] = cfg.floor_value;
                        }
                        if (!(ttot < dtf)) done = ST_OK;
                    }
                } else {
                    nfail++;
                    dt /= 2.0;
                    for (int i = 0; i < N; i++) y[i] = PREV[i];
                    if (dt / dtf < cfg.dt_ratio_floor) done = ST_DT_UNDERFLOW;
                }
                for (int i = 0; i < N; i++) Y[i] = y[i];
                if (done < 0 && !(cfg.sweep_budget > 0 && nsweeps >= cfg.sweep_budget)) {
                    substep_begin();
                } else if (MIXED && done == ST_OK && cfg.cons_tol != 0.0 && !F(F_FP64) &&
                           !conserved<Net>(io, cell, y, cfg.cons_tol)) {
                    /* start the cell again from its input, FP64 linear solves */
                    F(F_FP64) = 1;
                    if (!cell_begin(false)) {
                        cell_end(ST_OK);
                        qi = queue ? (long long)atomicAdd(queue, 1ull) : qi + stride;
                        fetch();
                    }
                } else {
                    if (done < 0) suspend();
                    else cell_end(done);
                    qi = queue ? (long long)atomicAdd(queue, 1ull) : qi + stride;
                    fetch();
                }
            }
            F(F_ACT) = active;
        }
        __syncthreads();
    }
}

}  // namespace dg
#endif
