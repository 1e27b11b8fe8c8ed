/*
 * Wide engine: one cell per CTA of 4 warps, for the last few stiff cells of
 * a hydro step (FP64 and mixed precision).
 *
 * The split engine (dg_split.cuh) gives each lane its own cell, which is
 * what a full GPU wants; but after the first launches of a step only a few
 * hundred stiff cells are left, each needing 10^4-10^5 more sequential
 * Newton sweeps, and a lone cell's sweep in the split engine runs its
 * elimination one row and one column after another on the 64-cycle FP64
 * issue of its warps' sub-partitions (measured with an instrumented copy: of
 * ~124k cycles per sweep, 44k in the LU row updates, 20k in the back
 * substitution).  Here the cell's 128 lanes share each phase instead:
 *   - temperature: the density and sum of n_i/(gamma-1) terms one per lane
 *     (generated term lists), T with log T and the bin on thread 0, Tge on
 *     warp 1;
 *   - the table interpolation, the residual, the Jacobian's scaling and
 *     the Newton update one entry per lane;
 *   - RHS rows and Jacobian entries that are flat sums of products: one
 *     term per lane from generated tables, then one sum per lane; the other
 *     rows and entries as generated scalar code on up to three warps
 *     meanwhile (networks without the tables: four scalar parts);
 *   - FP64 elimination: column j belongs to warp j mod 4; the owner of
 *     column k picks the pivot by a warp reduction and forms the
 *     multipliers one row per lane, then after one barrier every warp
 *     updates its own columns one entry per lane; rows stay in place
 *     (a row order records the interchanges);
 *   - back substitution on warp 0, lane i holding row i in registers.
 *
 * Mixed precision (the Newton matrix formed from FP64 products): the
 * equilibration exponents, the FP32 rounding and MixedSolve::factor's
 * elimination run one row, column or entry per lane of warp 0, the FP32
 * solves and the refinement steps on its lane 0, the FP64 refinement
 * residual one row per lane; the FP64 elimination above serves the systems
 * the split engine hands to it, and a converged cell that fails the
 * conservation check is re-solved from its input with FP64 solves.
 *
 * Every value is computed with exactly the split engine's operations in the
 * same order (the scaling of a Jacobian entry, the skip tests of the
 * elimination, dg_div with the pivot's reciprocal, the FP32 pivots and
 * fused multiply-adds, the printed expressions' products and sums), so the
 * results are bit-identical to it and, on the FP64 path, to the reference.
 * The kernel serves the resume launches of the stiff-cell redistribution
 * when at most cfg.wide_max cells were set aside (wide_tail per SM), CTA b
 * taking the b-th; otherwise it returns at once and the split engine's
 * launch does the work.
 */
#ifndef DG_WIDE_CUH
#define DG_WIDE_CUH

#include "dg_engine.cuh"

namespace dg {

/* A barrier among n threads of the CTA (named barrier id: bar.sync id, n),
 * called by every thread of the warps taking part; the host build supplies
 * its own. */
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ void dg_named_sync(int id, int n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
#elif !defined(DG_HOST_NAMED_SYNC)
__host__ __device__ inline void dg_named_sync(int, int) {}
#endif

/* Jacobian entries as the generated code produces them, before the scaling
 * of BE_Resid_Jac (applied afterwards, one entry per lane): put() stores the
 * value, zero() marks a structural zero. */
template <int N>
struct RawPut {
    double *J;
    int *Z;
    __device__ __forceinline__ void operator()(int q, int v, double jv) const
    {
        J[v * N + q] = jv;
        Z[v * N + q] = 0;
    }
    __device__ __forceinline__ void zero(int q, int v) const { Z[v * N + q] = 1; }
};

template <class Net, bool MIXED>
__global__ void __launch_bounds__(128, 3)
evolve_wide_kernel(CellIO io, TableSet ts, KernelCfg cfg, unsigned long long *queue)
{
    constexpr int N = Net::N;
    constexpr int NT = Net::NT;
    constexpr int NP = 4;
    static_assert(N <= 32, "the wide engine gives each row of the system a lane of one warp");
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    /* the mixed path with the Newton matrix in extended-range FP32 stays on
     * the split engine */
    if (!cfg.resume || !cfg.resume_count || cfg.wide_max <= 0 || (MIXED && cfg.jac_xf)) return;
    /* CTA b resumes the b-th set-aside cell: the launch has wide_max CTAs,
     * at least one per cell, and the first wave spreads them over the SMs */
    const unsigned int cnt = *cfg.resume_count;
    if (cnt > (unsigned int)cfg.wide_max || blockIdx.x >= cnt || blockIdx.x >= io.ncells) return;
    (void)queue;

    /* J: the Newton matrix, J[j * N + i] = row i, column j; MB, PRB:
     * multipliers and row order, double buffered by step; Z: structural
     * zeros of the Jacobian */
    __shared__ double J[N * N], R[NT], Y[N], G[N], U[N], U0[N], SC[N], INV[N], AT[N],
        RT[N], PREV[N], RPV[N], PV[N], XS[N], MB[2][N], S[6], TD[Net::T_ND], TQ[Net::T_NQ], TS[2];
    __shared__ int Z[N * N], FROW[N], PRB[2][N];
    __shared__ int s_act, s_okr, s_okj, s_bin, s_dense;
    /* sums of products (Net::SOP): the operands (rates first, so the
     * interpolation writes them there), the term values, and mdensity,
     * 1/mdensity and the ge row's and column's structural zeros */
    constexpr int NTV = Net::SOP_RT > Net::SOP_JT ? Net::SOP_RT : Net::SOP_JT;
    __shared__ double OPS[Net::SOP ? (Net::SOP_NOPS > NT ? Net::SOP_NOPS : NT) : 1],
        TV[Net::SOP ? NTV : 1], SMD[5];
    double *const Rp = Net::SOP ? OPS : R;
    /* mixed: FP32 factors, row and column scale exponents, FP32 pivot rows,
     * the refined solution and residual; s_mix 0 FP64 elimination, 1
     * refining, 2 refined, 3 stopped short; s_fp64: the cell is re-solved
     * with FP64 linear solves (it failed the conservation check) */
    __shared__ float JF[MIXED ? N * N : 1];
    __shared__ int SI[N], TJ[N], PXP[N];
    __shared__ double X[N], RR[N];
    __shared__ int s_mix, s_eprev, s_fp64;
    /* the solve's state after refinement step it is s_mixb[it & 1]: thread 0
     * writes the next step's slot while slower threads may still read this
     * step's */
    __shared__ int s_mixb[2];

    /* the species and their powers as operands (lanes), and the RHS's or
     * Jacobian's test for negative values (flag cleared on one) */
    auto sop_operands = [&](const double *y, int &okflag) {
        for (int i = tid; i < N; i += 128) {
            OPS[NT + i] = y[i];
            if (dg_lt0(y[i])) atomicAnd(&okflag, 0);
        }
        for (int k = tid; k < Net::SOP_NPOW; k += 128) {
            const double x = y[Net::sop_pow_sp(k)];
            double p;
            switch (Net::sop_pow_n(k)) {
            case 2: p = ::dg_ipow<2>(x); break;
            case 3: p = ::dg_ipow<3>(x); break;
            case 4: p = ::dg_ipow<4>(x); break;
            case 5: p = ::dg_ipow<5>(x); break;
            default: p = ::dg_ipow<6>(x); break;
            }
            OPS[NT + N + k] = p;
        }
    };

    /* thread-0 control state of the CTA's cell */
    long long cell = 0;
    double dtf = 0, dt = 0, ttot = 0;
    int siter = 0, isweep = 0, nsweeps = 0, nfail = 0;
    bool active = false, dense = false, fp64cell = false;

    auto substep_begin = [&]() {
        for (int i = 0; i < N; i++) {
            const double v = Y[i] * INV[i];
            U[i] = v;
            U0[i] = v;
            AT[i] = AT[i] * INV[i];
        }
        isweep = 0;
    };
    /* from_record: a set-aside cell, continued from its suspension record;
     * else (the mixed path's conservation re-solve) from the caller's input */
    auto cell_begin = [&](bool from_record) -> bool {
        if (!from_record) {
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
        }
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
        fp64cell = MIXED && rc[4 * N + 5] != 0.0;
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
        rc[4 * N + 5] = fp64cell ? 1.0 : 0.0;
        io.status[cell] = ST_SUSPENDED;
    };
    if constexpr (Net::SOP) {
        /* the constant operands, and the Jacobian's structural zeros off
         * the ge row and column (the tabled and scalar entries leave them) */
        for (int k = tid; k < Net::SOP_NLIT; k += 128) OPS[Net::SOP_LIT0 + k] = Net::sop_lit(k);
        if (tid == 0) OPS[Net::SOP_ONE] = 1.0;
        for (int e = tid; e < N * N; e += 128) {
            const int v = e / N, q = e - v * N;
            Z[e] = !Net::jraw(q, v) && q != Net::IGE && v != Net::IGE;
        }
    }
    if (tid == 0) {
        cell = (long long)io.order[blockIdx.x];
        active = cell >= 0 && cell_begin(true);
        if (cell >= 0 && !active) cell_end(ST_OK);
        s_act = active;
    }
    __syncthreads();
    while (s_act) {
        if (Net::T_LANES) {
            /* ---- P0a: the unscaled state (warp 0) and the temperature's
             *      terms, products on warp 0, quotients on warp 1 ---- */
            if (w == 0) {
                for (int i = l; i < N; i += 32) Y[i] = U[i] * SC[i];
                if (l < Net::T_ND) {
                    const int sp = Net::t_dsp(l);
                    TD[l] = Net::t_dw(l) * (U[sp] * SC[sp]);
                }
                if (l == 0) {
                    S[3] = -dt;
                    s_dense = dense || !(dt > 0.0);
                    s_okr = 1;
                    s_okj = 1;
                    s_mix = 0;
                    s_mixb[0] = 0;
                    s_fp64 = fp64cell;
                }
            } else if (w == 1 && l < Net::T_NQ) {
                const int sp = Net::t_qsp(l);
                TQ[l] = Net::t_quot(U[sp] * SC[sp]);
            }
            __syncthreads();
            /* ---- P0b: the two sums, in the printed order ---- */
            if (tid == 0) {
                double d = TD[0];
                for (int k = 1; k < Net::T_ND; k++) d = d + TD[k];
                TS[0] = d;
            } else if (tid == 32) {
                double q = TQ[0];
                for (int k = 1; k < Net::T_NQ; k++) q = q + TQ[k];
                TS[1] = q;
            }
            __syncthreads();
            /* ---- P0c: T, log T, bin (thread 0); Tge (warp 1) ---- */
            if (tid == 0) {
                const double T = Net::t_finish(TS[0], TS[1], Y[Net::IGE], ts.Tlo, ts.Thi);
                const double logT = dg_log(T);
                const int bin = (int)(ts.idbin * (logT - ts.lb));
                const int bc = bin <= 0 ? 0 : (bin >= ts.nbins ? ts.nbins - 1 : bin);
                const double t1 = (ts.lb + (bin) * ts.dbin);
                const double t2 = (ts.lb + (bin + 1) * ts.dbin);
                S[0] = T;
                S[2] = (logT - t1) / (t2 - t1);
                s_bin = bc;
            } else if (tid == 32) {
                S[1] = Net::tge_finish(TS[0], TS[1]);
            }
            __syncthreads();
        } else {
            /* ---- P0 (thread 0): unscale, temperature, bin ---- */
            if (tid == 0) {
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
                S[3] = -dt;
                s_bin = bc;
                s_dense = dense || !(dt > 0.0);
                s_okr = 1;
                s_okj = 1;
                s_mix = 0;
                s_mixb[0] = 0;
                s_fp64 = fp64cell;
            }
            __syncthreads();
        }
        /* ---- P1: interpolation, one table per lane ---- */
        for (int k = tid; k < NT; k += 128) {
            if (Net::zdep(k)) {
                Rp[k] = ts.zvals[k];
            } else {
                const double2 pr = __ldg(ts.pairs + (size_t)s_bin * NT + k);
                Rp[k] = pr.x + S[2] * pr.y;
            }
        }
        __syncthreads();
        if constexpr (Net::SOP) {
            /* ---- P2a: the species and their powers as operands; any
             *      negative value fails the RHS ---- */
            sop_operands(Y, s_okr);
            if (Net::SOP_RMD && tid == 96) SMD[0] = Net::mdensity_of(Y);
            __syncthreads();
            /* ---- P2b: warps [0, SOP_RK) the scalar rows, lane 0 each;
             *      the other warps every term, one per lane, then every
             *      tabled row's sum, one per lane ---- */
            if (w < Net::SOP_RK) {
                if (l == 0) {
                    double y[N], f[N];
                    for (int i = 0; i < N; i++) y[i] = Y[i];
                    const Slots<1> Rs{Rp};
                    bool ok = true;
                    switch (w) {
                    case 0: ok = Net::template rhs_rest<0>(y, Rs, S[0], ts.z, f); break;
                    case 1: ok = Net::template rhs_rest<1>(y, Rs, S[0], ts.z, f); break;
                    default: ok = Net::template rhs_rest<2>(y, Rs, S[0], ts.z, f); break;
                    }
                    if (ok) {
                        for (int i = 0; i < N; i++)
                            if (Net::sop_rpart(i) == w) G[i] = f[i];
                    } else {
                        atomicAnd(&s_okr, 0);
                    }
                }
            } else {
                constexpr int NW = 4 - Net::SOP_RK;
                const int sl = tid - 32 * Net::SOP_RK;
                for (int t = sl; t < Net::SOP_RT; t += 32 * NW) {
                    const int o0 = Net::sop_rterm(t, 0);
                    double v = OPS[o0 & 0x7fff];
                    for (int f = 1; f < Net::SOP_FMAX; f++) v = v * OPS[Net::sop_rterm(t, f)];
                    TV[t] = (o0 & 0x8000) ? -v : v;
                }
                if (NW == 1) __syncwarp();
                else dg_named_sync(1, 32 * NW);
                for (int e = sl; e < Net::SOP_RE; e += 32 * NW) {
                    int row, t0, t1, post;
                    Net::sop_rentry(e, row, t0, t1, post);
                    double acc = TV[t0];
                    for (int t = t0 + 1; t < t1; t++) acc = acc + TV[t];
                    if (post & 1) acc = acc / SMD[0];
                    G[row] = acc;
                }
            }
        } else if (l == 0) {
            /* ---- P2: RHS rows of part w (lane 0 of warp w) ---- */
            double y[N], f[N];
            for (int i = 0; i < N; i++) y[i] = Y[i];
            const Slots<1> Rs{Rp};
            bool ok = true;
            switch (w) {
            case 0: ok = Net::template rhs<NP, 0>(y, Rs, S[0], ts.z, f); break;
            case 1: ok = Net::template rhs<NP, 1>(y, Rs, S[0], ts.z, f); break;
            case 2: ok = Net::template rhs<NP, 2>(y, Rs, S[0], ts.z, f); break;
            default: ok = Net::template rhs<NP, 3>(y, Rs, S[0], ts.z, f); break;
            }
            if (ok) {
                for (int i = 0; i < N; i++)
                    if (Net::rhs_row_part(NP, i) == w) G[i] = f[i];
            } else {
                atomicAnd(&s_okr, 0);
            }
        }
        __syncthreads();
        /* ---- P3: residual g = u - u0 - dt f (scaled), one row per lane ---- */
        if (s_okr) for (int i = tid; i < N; i += 128) {
            const double dtv = -S[3];
            const double u = Y[i] * INV[i];
            double g = G[i] * INV[i];
            g = u - U0[i] - dtv * g;
            G[i] = g;
            U[i] = u;
            Y[i] = u * SC[i];
        }
        __syncthreads();
        const bool do_j = s_okr != 0;
        if constexpr (Net::SOP) {
            /* ---- P4a: operands from the Jacobian's state; mdensity and
             *      what the ge row and column need ---- */
            if (do_j) {
                sop_operands(Y, s_okj);
                if (tid == 96) {
                    const double md = Net::mdensity_of(Y);
                    SMD[1] = md;
                    SMD[2] = 1.0 / md;
                    SMD[3] = dg_quot(0.0, md);
                    SMD[4] = 0.0 * S[1];
                }
            }
            __syncthreads();
            /* ---- P4b: scalar entries on warps [0, SOP_JK), terms and
             *      sums on the others, the ge zeros ---- */
            if (do_j) {
                if (w < Net::SOP_JK) {
                    if (l == 0) {
                        double y[N];
                        for (int i = 0; i < N; i++) y[i] = Y[i];
                        const Slots<1> Rs{Rp};
                        const RawPut<N> put{J, Z};
                        bool ok = true;
                        switch (w) {
                        case 0: ok = Net::template jac_rest<0>(y, Rs, S[1], S[0], ts.z, put); break;
                        case 1: ok = Net::template jac_rest<1>(y, Rs, S[1], S[0], ts.z, put); break;
                        default: ok = Net::template jac_rest<2>(y, Rs, S[1], S[0], ts.z, put); break;
                        }
                        if (!ok) atomicAnd(&s_okj, 0);
                    }
                } else {
                    constexpr int NW = 4 - Net::SOP_JK;
                    const int sl = tid - 32 * Net::SOP_JK;
                    for (int t = sl; t < Net::SOP_JT; t += 32 * NW) {
                        const int o0 = Net::sop_jterm(t, 0);
                        double v = OPS[o0 & 0x7fff];
                        for (int f = 1; f < Net::SOP_FMAX; f++) v = v * OPS[Net::sop_jterm(t, f)];
                        TV[t] = (o0 & 0x8000) ? -v : v;
                    }
                    if (NW == 1) __syncwarp();
                    else dg_named_sync(2, 32 * NW);
                    const double md = SMD[1], rmd = SMD[2], Tge = S[1];
                    for (int e = sl; e < Net::SOP_JE; e += 32 * NW) {
                        int q, v, t0, t1, post;
                        Net::sop_jentry(e, q, v, t0, t1, post);
                        double acc = TV[t0];
                        for (int t = t0 + 1; t < t1; t++) acc = acc + TV[t];
                        if (post & 1) acc = dg_div(acc, md, rmd);
                        if (post & 2) acc = acc * Tge;
                        J[v * N + q] = acc;
                    }
                    /* the ge row's and column's structural zeros: 0/mdensity,
                     * 0*Tge, and their product on the diagonal */
                    for (int i = sl; i < N; i += 32 * NW) {
                        if (!Net::jraw(Net::IGE, i))
                            J[i * N + Net::IGE] = i == Net::IGE ? SMD[3] * Tge : SMD[3];
                        if (i != Net::IGE && !Net::jraw(i, Net::IGE)) J[Net::IGE * N + i] = SMD[4];
                    }
                }
            }
        } else if (do_j && l == 0) {
            /* ---- P4: Jacobian entries of part w (lane 0 of warp w), raw ---- */
            double y[N];
            for (int i = 0; i < N; i++) y[i] = Y[i];
            const Slots<1> Rs{Rp};
            const RawPut<N> put{J, Z};
            bool ok = true;
            switch (w) {
            case 0: ok = Net::template jac<NP, 0>(y, Rs, S[1], S[0], ts.z, put); break;
            case 1: ok = Net::template jac<NP, 1>(y, Rs, S[1], S[0], ts.z, put); break;
            case 2: ok = Net::template jac<NP, 2>(y, Rs, S[1], S[0], ts.z, put); break;
            default: ok = Net::template jac<NP, 3>(y, Rs, S[1], S[0], ts.z, put); break;
            }
            if (!ok) atomicAnd(&s_okj, 0);
        }
        __syncthreads();
        const bool do_lu = do_j && s_okj;
        /* ---- P4b: BE_Resid_Jac's scaling, one entry per lane (JacPut's
         *      operations), u = y / scale, the identity row order ---- */
        if (do_lu) {
            const double mdt = S[3];
            for (int e = tid; e < N * N; e += 128) {
                const int v = e / N, q = e - v * N;
                if (Z[e] && !s_dense) {
                    J[e] = (q == v) ? 1.0 : -0.0;
                } else {
                    double a = (Z[e] ? 0.0 : J[e]) * INV[q];
                    a = a * SC[v];
                    a = mdt * a;
                    if (q == v) a = a + 1.0;
                    J[e] = a;
                }
            }
            for (int i = tid; i < N; i += 128) {
                U[i] = Y[i] * INV[i];
                PRB[0][i] = i;
            }
        }
        __syncthreads();   /* the whole matrix, for the first pivot column's owner or the
                              mixed solve's warp */
        /* ---- P5 (mixed): the equilibrated FP32 factorisation on warp 0
         *      (one row, column or entry per lane, MixedSolve's operations),
         *      its solves and the FP64 refinement on lane 0 of warp 0, the
         *      refinement residual one row per lane; the FP64 elimination
         *      below for a dense or non-finite system, a cell that is being
         *      re-solved in FP64, or a refinement that stopped short ---- */
        bool lu64 = do_lu;
        if constexpr (MIXED) {
            using MS = MixedSolve<Net, 1>;
            const MS ms{Slots<1>{J}, SlotsF<1>{JF}};
            const bool eq = do_lu && !s_dense && !s_fp64;
            if (eq && w == 0) {
                /* row scale exponents and the finiteness of A and g */
                bool fin = true;
                if (l < N) {
                    int m = 0;
                    fin = dg_expo(G[l]) != 0x7ff;
                    for (int j = 0; j < N; j++) {
                        const int e = dg_expo(J[j * N + l]);
                        fin = fin && e != 0x7ff;
                        m = e > m ? e : m;
                    }
                    SI[l] = m ? 1022 - m : 0;
                }
                const bool allfin = __all_sync(0xffffffffu, fin);
                __syncwarp();
                /* column scale exponents */
                if (l < N) {
                    int cm = MS::NONE;
                    for (int i = 0; i < N; i++) {
                        if (!Net::jnz(i, l)) continue;
                        const int e = dg_expo(J[l * N + i]);
                        if (e != 0 && e + SI[i] > cm) cm = e + SI[i];
                    }
                    TJ[l] = cm == MS::NONE ? 0 : 1022 - cm;
                }
                __syncwarp();
                if (allfin) {
                    /* R A C rounded to FP32 */
                    for (int e = l; e < N * N; e += 32) {
                        const int j = e / N, i = e - j * N;
                        JF[e] = Net::jnz(i, j) ? dg_f32_scaled(J[e], SI[i] + TJ[j]) : 0.0f;
                    }
                    __syncwarp();
                    /* MixedSolve::factor, one row / entry per lane */
                    for (int k = 0; k < N - 1; k++) {
                        const bool cand = l >= k && l < N;
                        const unsigned int key = cand ? __float_as_uint(fabsf(JF[k * N + l])) : 0u;
                        const unsigned int kk = __shfl_sync(0xffffffffu, key, k);
                        int p = k;
                        if (kk <= 0x7f800000u) {
                            /* the first row of largest |a| among the non-NaN ones */
                            const bool valid = cand && key <= 0x7f800000u;
                            const unsigned int mx = __reduce_max_sync(0xffffffffu, valid ? key : 0u);
                            p = __ffs(__ballot_sync(0xffffffffu, valid && key == mx)) - 1;
                        }
                        if (p != k && l >= k && l < N) {
                            const float t = JF[l * N + k];
                            JF[l * N + k] = JF[l * N + p];
                            JF[l * N + p] = t;
                        }
                        if (l == 0) PXP[k] = p;
                        __syncwarp();
                        const float rp = 1.0f / JF[k * N + k];
                        const float mi = l > k && l < N ? JF[k * N + l] * rp : 0.0f;
                        __syncwarp();
                        if (l > k && l < N) JF[k * N + l] = mi;
                        if (l == 0) JF[k * N + k] = rp;
                        __syncwarp();
                        const int rows = N - 1 - k;
                        for (int e = l; e < rows * rows; e += 32) {
                            const int j = k + 1 + e / rows, i = k + 1 + e % rows;
                            JF[j * N + i] = fmaf(-JF[k * N + i], JF[j * N + k], JF[j * N + i]);
                        }
                        __syncwarp();
                    }
                    if (l == 0) {
                        PXP[N - 1] = N - 1;
                        JF[(N - 1) * N + (N - 1)] = 1.0f / JF[(N - 1) * N + (N - 1)];
                        /* the first solve */
                        double g[N], x[N];
                        int sx[N], tx[N], px[N];
                        for (int i = 0; i < N; i++) {
                            g[i] = G[i];
                            sx[i] = SI[i];
                            tx[i] = TJ[i];
                            px[i] = PXP[i];
                        }
                        int ed;
                        if (ms.apply(px, sx, tx, g, x, ed)) {
                            for (int i = 0; i < N; i++) X[i] = x[i];
                            s_mixb[0] = 1;
                            s_eprev = 0x7ff;
                        }
                    }
                }
            }
            __syncthreads();
            int it = 0;
            for (; it < MS::MAX_REFINE; it++) {
                if (!(eq && s_mixb[it & 1] == 1)) break;
                if (w == 0) {
                    if (l < N) RR[l] = ms.residual_row(l, G[l], X);
                    __syncwarp();
                    if (l == 0) {
                        double r[N], x[N];
                        int sx[N], tx[N], px[N];
                        for (int i = 0; i < N; i++) {
                            r[i] = RR[i];
                            x[i] = X[i];
                            sx[i] = SI[i];
                            tx[i] = TJ[i];
                            px[i] = PXP[i];
                        }
                        int eprev = s_eprev, next = 0;
                        bool more;
                        if (ms.refine(px, sx, tx, r, x, eprev, more)) {
                            for (int i = 0; i < N; i++) X[i] = x[i];
                            s_eprev = eprev;
                            next = more ? 1 : 2;
                            if (DG_MIXED_STRICT && !more && !MS::refined(x, eprev)) next = 3;
                        }
                        s_mixb[(it + 1) & 1] = next;
                    }
                }
                __syncthreads();
            }
            /* a refinement that ran out of steps or stopped short of 2^-40
             * goes to the FP64 elimination */
            if (tid == 0) {
                int m = eq ? s_mixb[it & 1] : 0;
                if (DG_MIXED_STRICT && (m == 1 || m == 3)) m = 0;
                s_mix = m;
            }
            __syncthreads();
            if (eq && s_mix != 0)
                for (int i = tid; i < N; i += 128) XS[i] = X[i];
            lu64 = do_lu && s_mix == 0;
        }
        /* ---- P5: Gauss_Elim with one barrier per elimination step.
         * Column j belongs to warp j mod 4 throughout.  Step k: the owner of
         * column k finds the pivot (a warp reduction that picks the first
         * row of largest magnitude, as the serial scan), records the row
         * interchange in the row order (the rows stay in place: logical row
         * i is J row PR[i]) and forms the multipliers a_ik / pivot, one row
         * per lane; after the barrier every warp updates its own columns,
         * one (row, column) entry per lane, one warp the right-hand side,
         * another the pivot's reciprocal for the back substitution.  The
         * owner of column k+1 has just updated that column itself and goes
         * on to step k+1 at once; the row order and the multipliers are
         * double-buffered for the warps still in step k. ---- */
        for (int k = 0; k < N - 1; k++) {
            const int *PRo = PRB[k & 1];
            int *PRn = PRB[(k + 1) & 1];
            double *M = MB[k & 1];
            if (lu64 && w == (k & 3)) {
                const int i = l;
                const bool cand = i >= k && i < N;
                const int pri = i < N ? PRo[i] : 0;
                const double a = cand ? J[k * N + pri] : 0.0;
                const unsigned long long key = dg_bits(a) << 1;
                const bool valid = cand && key <= DG_INF2;
                const double ak = __shfl_sync(0xffffffffu, a, k);
                const int prk = __shfl_sync(0xffffffffu, pri, k);
                int p = k;
                if ((dg_bits(ak) << 1) <= DG_INF2) {
                    /* largest |a| among the finite candidates, first row on a tie */
                    const unsigned int hi = valid ? (unsigned int)(key >> 32) : 0u;
                    const unsigned int mhi = __reduce_max_sync(0xffffffffu, hi);
                    const bool c1 = valid && hi == mhi;
                    const unsigned int lo = c1 ? (unsigned int)key : 0u;
                    const unsigned int mlo = __reduce_max_sync(0xffffffffu, lo);
                    p = __ffs(__ballot_sync(0xffffffffu, c1 && (unsigned int)key == mlo)) - 1;
                }
                const double piv = __shfl_sync(0xffffffffu, a, p);
                const int prp = __shfl_sync(0xffffffffu, pri, p);
                /* logical row p now holds the old row k (and its a_kk) */
                const int r = i == k ? prp : (i == p ? prk : pri);
                if (i < N) PRn[i] = r;
                if (i > k && i < N) {
                    const double m = dg_quot(i == p ? ak : a, piv);
                    J[k * N + r] = m;
                    M[i] = m;
                }
                if (l == 0) PV[k] = piv;
                __syncwarp();
            }
            __syncthreads();
            if (lu64) {
                const int pk = PRn[k];
                /* row k's entries right of the pivot all finite? */
                bool fin = true;
                for (int j = k + 1 + l; j < N; j += 32) fin = fin && dg_finite(J[j * N + pk]);
                const bool rowfin = __all_sync(0xffffffffu, fin);
                const int rows = N - 1 - k;
                const int j0 = k + 1 + ((w - (k + 1)) & 3);
                const int ncol = j0 < N ? (N - 1 - j0) / 4 + 1 : 0;
                for (int e = l; e < ncol * rows; e += 32) {
                    const int c = e / rows, i = k + 1 + (e - c * rows), j = j0 + 4 * c;
                    const double m = M[i];
                    if (dg_nonzero(m) || !rowfin) {
                        const double akj = J[j * N + pk];
                        if (dg_nonzero(akj) || !dg_finite(m)) {
                            const int r = PRn[i];
                            J[j * N + r] = J[j * N + r] - m * akj;
                        }
                    }
                }
                if (w == ((k + 2) & 3)) {
                    const double xk = G[pk];
                    for (int i = k + 1 + l; i < N; i += 32) {
                        const double m = M[i];
                        if (dg_nonzero(m) || !dg_finite(xk)) G[PRn[i]] = G[PRn[i]] - m * xk;
                    }
                }
                if (w == ((k + 3) & 3) && l == 0) RPV[k] = 1.0 / PV[k];
                __syncwarp();
            }
        }
        __syncthreads();
        /* ---- back substitution (warp 0, lane i = row i, in registers):
         * lane j forms x_j from its row's products in increasing column
         * order, a shuffle hands x_j to the warp, and every row above forms
         * its product with x_j at once ---- */
        if (lu64 && w == 0) {
            const int *PRf = PRB[(N - 1) & 1];
            const int rl = l < N ? PRf[l] : 0;
            double a[N], p[N];
#pragma unroll
            for (int t = 0; t < N; t++) {
                a[t] = l < N ? J[t * N + rl] : 0.0;
                p[t] = 0.0;
            }
            const double g0 = l < N ? G[rl] : 0.0;
            unsigned int f = 0;   /* bit t: row l subtracts its product with x_t */
            double xv = 0.0;
#pragma unroll
            for (int j = N - 1; j >= 0; j--) {
                if (l == j) {
                    double acc = g0;
#pragma unroll
                    for (int t = j + 1; t < N; t++)
                        if (f & (1u << t)) acc = acc - p[t];
                    xv = j == N - 1 ? dg_quot(acc, a[j]) : dg_div(acc, a[j], RPV[j]);
                    XS[j] = xv;
                }
                const double xj = __shfl_sync(0xffffffffu, xv, j);
                if (l < j) {
                    p[j] = a[j] * xj;
                    if (dg_nonzero(a[j]) || !dg_finite(xj)) f |= 1u << j;
                }
            }
        }
        __syncthreads();
        /* ---- P6a: Newton update and each row's max-norm / NaN test ---- */
        if (s_okr && s_okj) for (int i = tid; i < N; i += 128) {
            const double u = U[i] - 1.0 * XS[i];
            U[i] = u;
            FROW[i] = dg_abs_gt_val(XS[i], AT[i] + RT[i] * fabs(u)) ? 1 : (dg_isnan(u) ? 2 : 0);
        }
        __syncthreads();
        /* ---- P6b (thread 0): the first row that fails decides, as in the
         *      reference's row loop; substep control ---- */
        if (tid == 0) {
            bool ok = s_okr && s_okj, unsolved = false, nan = false;
            if (ok) {
                for (int i = 0; i < N; i++) {
                    const int r = FROW[i];
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
                } else if (MIXED && done == ST_OK && cfg.cons_tol != 0.0 && !fp64cell &&
                           !conserved<Net>(io, cell, y, cfg.cons_tol)) {
                    /* start the cell again from its input, FP64 linear solves */
                    fp64cell = true;
                    if (!cell_begin(false)) {
                        cell_end(ST_OK);
                        active = false;
                    }
                } else {
                    if (done < 0) suspend();
                    else cell_end(done);
                    active = false;
                }
            }
            s_act = active;
        }
        __syncthreads();
    }
}

}  // namespace dg
#endif
