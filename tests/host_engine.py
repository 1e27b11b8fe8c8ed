"""The single-lane CUDA engine (dengo_gb300/csrc/dg_engine.cuh, evolve_kernel)
compiled for the host, for tests that need no GPU.

The kernel source is compiled unchanged with g++ against CUDA's host headers;
the few device built-ins it uses are given host meanings: ``threadIdx`` /
``blockIdx`` / ``gridDim`` are set by the driver below, which runs the 32
lanes of one CTA one after another; ``atomicAdd`` is a plain add (one lane
runs at a time); ``__shfl_sync`` hands lane 0's value to the later lanes (lane
0 runs first); ``__ldg`` is a load; the FP32 bit casts and ``__clz`` are
their definitions.  IEEE double and single arithmetic, ``fma`` and ``fmaf``
round the same way on the host as on the GPU (the CUDA build uses
``--fmad=false``, this one ``-ffp-contract=off``), so every cell's result is
the device's.  Which lane takes which cell differs from the GPU; no cell's
result depends on that.

``hx_evolve`` is one solve of a batch of cells (AoS, mass densities + ge)
through the same launches as ``<n>_solve_cells_device``: one launch, or with
a sweep budget the three launches of the stiff-cell redistribution, the
resume list built on the host.

The split engine (dg_split.cuh, evolve_split_kernel: 32 cells per CTA, each
cell's sweep shared by NP warps that meet at __syncthreads) is built the
same way with ``engine="split"``, but its 32 x NP lanes run as that many host
threads: ``__syncthreads`` is a barrier across them, ``__syncthreads_or`` a
reduction between barriers, the warp collectives (``__shfl_sync``,
``__ballot_sync``, ``__all_sync``, ``__reduce_max_sync``, ``__syncwarp``)
barriers across the warp's 32 threads around a value each posts, and the
atomics take a lock.  One CTA runs the whole batch from the work queue.  A build that hangs is cut off by the caller's timeout
(``evolve_in_subprocess``).  ``engine="wide"`` adds the wide engine
(dg_wide.cuh, one CTA of 128 threads per cell) and hands it every cell of
the resume launches.
"""
import ctypes as C
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dengo_gb300", "csrc")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
P_D = C.POINTER(C.c_double)
P_I = C.POINTER(C.c_int)

PRELUDE = r'''
#include <math.h>
#include <string.h>
#include <vector>
#include <cuda_runtime.h>
struct hx_dim3 { unsigned x, y, z; };
static hx_dim3 threadIdx, blockIdx, gridDim, blockDim;
static inline float __uint_as_float(unsigned int u) { float f; memcpy(&f, &u, 4); return f; }
static inline unsigned int __float_as_uint(float f) { unsigned int u; memcpy(&u, &f, 4); return u; }
static inline int __clz(unsigned int x) { return x ? __builtin_clz(x) : 32; }
static inline double __fma_rn(double a, double b, double c) { return fma(a, b, c); }
static inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v)
{
    const unsigned long long o = *p;
    *p += v;
    return o;
}
static unsigned long long hx_lane0;
static inline unsigned long long __shfl_sync(unsigned, unsigned long long v, int)
{
    if ((threadIdx.x & 31) == 0) hx_lane0 = v;
    return hx_lane0;
}
template <class T> static inline T __ldg(const T *p) { return *p; }
#define __launch_bounds__(...)
namespace dg { double dg_smem[1 << 16]; }  /* the CTA's dynamic shared memory */
#include "dg_engine.cuh"
'''

PRELUDE_SPLIT = r'''
#include <math.h>
#include <string.h>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>
#include <cuda_runtime.h>
struct hx_dim3 { unsigned x, y, z; };
static thread_local hx_dim3 threadIdx;
static hx_dim3 blockIdx, gridDim, blockDim;
static inline float __uint_as_float(unsigned int u) { float f; memcpy(&f, &u, 4); return f; }
static inline unsigned int __float_as_uint(float f) { unsigned int u; memcpy(&u, &f, 4); return u; }
static inline int __clz(unsigned int x) { return x ? __builtin_clz(x) : 32; }
static inline double __fma_rn(double a, double b, double c) { return fma(a, b, c); }
static std::mutex hx_atomic_lock;
template <class T> static inline T atomicAdd(T *p, T v)
{
    std::lock_guard<std::mutex> g(hx_atomic_lock);
    const T o = *p;
    *p += v;
    return o;
}
static inline int atomicAnd(int *p, int v)
{
    std::lock_guard<std::mutex> g(hx_atomic_lock);
    const int o = *p;
    *p = o & v;
    return o;
}
static inline int atomicMax(int *p, int v)
{
    std::lock_guard<std::mutex> g(hx_atomic_lock);
    const int o = *p;
    if (v > o) *p = v;
    return o;
}
static inline int atomicMin(int *p, int v)
{
    std::lock_guard<std::mutex> g(hx_atomic_lock);
    const int o = *p;
    if (v < o) *p = v;
    return o;
}
/* A reusable barrier.  Waiters yield the core for a while (the lanes far
 * outnumber the host's cores, and most barriers are met quickly), then
 * sleep on the generation counter, so that threads parked at one barrier
 * (the other warps, while one warp runs a long stretch of warp-level steps)
 * do not crowd out the threads that are working. */
struct hx_barrier {
    explicit hx_barrier(int n) : count(n), left(n), gen(0) {}
    void arrive_and_wait()
    {
        const unsigned g = gen.load(std::memory_order_acquire);
        if (left.fetch_sub(1, std::memory_order_acq_rel) == 1) {
            left.store(count, std::memory_order_relaxed);
            gen.store(g + 1, std::memory_order_release);
            gen.notify_all();
        } else {
            for (int spin = 0; spin < 64; spin++) {
                if (gen.load(std::memory_order_acquire) != g) return;
                std::this_thread::yield();
            }
            while (gen.load(std::memory_order_acquire) == g) gen.wait(g, std::memory_order_acquire);
        }
    }
    const int count;
    std::atomic<int> left;
    std::atomic<unsigned> gen;
};
static hx_barrier *hx_cta;      /* all lanes of the CTA */
static hx_barrier *hx_warp[32];  /* the 32 lanes of each warp */
/* named barriers (bar.sync id, n): made by their first caller */
static hx_barrier *hx_named[16];
static std::mutex hx_named_lock;
#define DG_HOST_NAMED_SYNC
namespace dg {
static void dg_named_sync(int id, int n)
{
    hx_barrier *b;
    {
        std::lock_guard<std::mutex> g(hx_named_lock);
        if (!hx_named[id]) hx_named[id] = new hx_barrier(n);
        b = hx_named[id];
    }
    b->arrive_and_wait();
}
}
/* A CTA of `threads` lanes (a multiple of 32): its barrier and one per warp. */
static void hx_setup(int threads)
{
    static std::vector<hx_barrier *> keep;
    for (hx_barrier *b : keep) delete b;
    keep.clear();
    for (int i = 0; i < 16; i++) {
        if (hx_named[i]) keep.push_back(hx_named[i]);
        hx_named[i] = nullptr;
    }
    hx_cta = new hx_barrier(threads);
    keep.push_back(hx_cta);
    for (int w = 0; w < (threads + 31) / 32; w++) {
        hx_warp[w] = new hx_barrier(32);
        keep.push_back(hx_warp[w]);
    }
}
static inline void __syncthreads() { hx_cta->arrive_and_wait(); }
static std::atomic<int> hx_or;
static inline int __syncthreads_or(int p)
{
    hx_cta->arrive_and_wait();
    if (threadIdx.x == 0) hx_or = 0;
    hx_cta->arrive_and_wait();
    if (p) hx_or |= 1;
    hx_cta->arrive_and_wait();
    return hx_or.load();
}
/* Warp collectives, called by all 32 lanes of a warp: each lane posts its
 * value, the warp meets, each reads what it needs, the warp meets again. */
static unsigned long long hx_wbuf[32][32];
static inline void __syncwarp(unsigned = 0xffffffffu) { hx_warp[threadIdx.x >> 5]->arrive_and_wait(); }
static inline unsigned long long *hx_post(unsigned long long b)
{
    const int w = threadIdx.x >> 5;
    hx_wbuf[w][threadIdx.x & 31] = b;
    hx_warp[w]->arrive_and_wait();
    return hx_wbuf[w];
}
template <class T> static inline T __shfl_sync(unsigned, T v, int src)
{
    unsigned long long b = 0;
    memcpy(&b, &v, sizeof(T));
    const unsigned long long r = hx_post(b)[src & 31];
    __syncwarp();
    T o;
    memcpy(&o, &r, sizeof(T));
    return o;
}
static inline unsigned __ballot_sync(unsigned, int p)
{
    const unsigned long long *v = hx_post(p != 0);
    unsigned m = 0;
    for (int i = 0; i < 32; i++) m |= (unsigned)(v[i] != 0) << i;
    __syncwarp();
    return m;
}
static inline int __all_sync(unsigned, int p) { return __ballot_sync(~0u, p) == 0xffffffffu; }
static inline unsigned __reduce_max_sync(unsigned, unsigned x)
{
    const unsigned long long *v = hx_post(x);
    unsigned m = 0;
    for (int i = 0; i < 32; i++) m = (unsigned)v[i] > m ? (unsigned)v[i] : m;
    __syncwarp();
    return m;
}
static inline int __ffs(int x) { return __builtin_ffs(x); }
template <class T> static inline T __ldg(const T *p) { return *p; }
#define __launch_bounds__(...)
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif
namespace dg { double dg_smem[1 << 16]; }  /* the CTA's dynamic shared memory */
%(kernel_source)s
'''

DRIVER_SPLIT_LAUNCH = r'''
constexpr int NP = 4;
template <bool MIXED>
static void launch(dg::CellIO io, dg::TableSet ts, dg::KernelCfg cfg, unsigned long long *queue)
{
    static_assert(dg::SplitLayout<Net, NP, MIXED>::bytes() <= sizeof(dg::dg_smem), "shared memory");
    blockIdx.x = 0;
    gridDim.x = 1;
    blockDim.x = 32 * NP;
    hx_setup(32 * NP);
    std::vector<std::thread> lanes;
    for (unsigned t = 0; t < 32 * NP; t++)
        lanes.emplace_back([=]() {
            threadIdx.x = t;
            dg::evolve_split_kernel<Net, NP, MIXED>(io, ts, cfg, queue);
        });
    for (auto &th : lanes) th.join();
}
'''

DRIVER_WIDE_LAUNCH = DRIVER_SPLIT_LAUNCH.replace("static void launch(", "static void launch_split(") + r'''
/* The split engine, and for the resume launches the wide engine
 * (dg_wide.cuh, one CTA of 4 warps per cell) with every set-aside cell:
 * the split engine's launch then returns at once (not for the Newton matrix
 * in extended-range FP32). */
template <bool MIXED>
static void launch(dg::CellIO io, dg::TableSet ts, dg::KernelCfg cfg, unsigned long long *queue)
{
    const bool wide = cfg.resume && !cfg.jac_xf;
    if (wide) cfg.wide_max = 1 << 30;
    launch_split<MIXED>(io, ts, cfg, queue);
    if (!wide) return;
    /* one CTA per set-aside cell, one after another */
    const unsigned int count = *cfg.resume_count;
    for (unsigned int b = 0; b < count; b++) {
        blockIdx.x = b;
        gridDim.x = count;
        blockDim.x = 128;
        hx_setup(128);
        std::vector<std::thread> lanes;
        for (unsigned t = 0; t < 128; t++)
            lanes.emplace_back([=]() {
                threadIdx.x = t;
                dg::evolve_wide_kernel<Net, MIXED>(io, ts, cfg, queue);
            });
        for (auto &th : lanes) th.join();
    }
}
'''

DRIVER_LANE_LAUNCH = r'''
template <bool MIXED>
static void launch(dg::CellIO io, dg::TableSet ts, dg::KernelCfg cfg, unsigned long long *queue)
{
    constexpr int B = 32;
    static_assert(dg::Lane<Net, B, MIXED>::SLOTS * B <= (1 << 16), "host shared memory");
    blockIdx.x = 0;
    gridDim.x = 1;
    blockDim.x = B;
    for (unsigned t = 0; t < B; t++) {
        threadIdx.x = t;
        dg::evolve_kernel<Net, B, MIXED>(io, ts, cfg, queue);
    }
}
'''

DRIVER_STRIP = r'''
using Net = dgnet_%(name)s::Net;
constexpr int NN = Net::N;
constexpr int NT = Net::NT;

/* <n>_run_strip (dg_api.cuh): the Cython driver's loop on one strip of
 * number densities, one CTA of ceil(nstrip / 32) x 32 lanes. */
extern "C" int hx_run_strip(double *input, const double *rtol, double *atol, int nstrip,
                            double tf, int niter, double z, const double *const *tables,
                            double *ttot, double *dt, double *traj, double *traj_T,
                            unsigned char *traj_ok, double *traj_t, double *traj_dt)
{
    static Net::Data data;
    Net::setup_bins(&data);
    const int nbins = Net::NT_LEN - 1;
    std::vector<double2> pairs((size_t)nbins * NT);
    for (int b = 0; b < nbins; b++)
        for (int k = 0; k < NT; k++)
            pairs[(size_t)b * NT + k] = make_double2(tables[k][b], tables[k][b + 1] - tables[k][b]);
    dg::TableSet ts{pairs.data(), nbins, log(data.bounds[0]), data.dbin, data.idbin,
                    data.bounds[0], data.bounds[1], z, {}};
    double sc[3] = {0, 0, 0};
    int iters[16] = {0};
    dg::RunOut o{};
    o.ttot = sc;
    o.dt = sc + 1;
    o.iters = iters;
    o.traj = traj;
    o.traj_T = traj_T;
    o.traj_ok = traj_ok;
    o.traj_t = traj_t;
    o.traj_dt = traj_dt;
    const int threads = ((nstrip + 31) / 32) * 32;
    blockIdx.x = 0;
    gridDim.x = 1;
    blockDim.x = threads;
    hx_setup(threads);
    std::vector<std::thread> lanes;
    for (int t = 0; t < threads; t++)
        lanes.emplace_back([=]() {
            threadIdx.x = t;
            dg::run_strip_kernel<Net>(input, rtol, atol, nstrip, tf, niter, ts, 10, o);
        });
    for (auto &th : lanes) th.join();
    *ttot = sc[0];
    *dt = sc[1];
    return iters[0];
}

/* dengo_evolve_<n> in lockstep (evolve_lockstep_kernel) on one strip of at
 * most 1024 cells (AoS, mass densities + ge), launch after launch as the
 * library runs it; with dump the kernel stops after every accepted substep
 * and each of its dumps (prev, T, time, timestep, substep number) is
 * appended to the output arrays (max_dumps of them).  Returns the number of
 * dumps; *dt in: the initial step (< 0: dtf/1e5), out: the last. */
extern "C" int hx_evolve_lockstep(double *input, const double *rtol, double *atol, int dims,
                                  double dtf, double *dt, double z, const double *const *tables,
                                  int dump, int max_dumps, double *d_species, double *d_T,
                                  double *d_time, double *d_dt, int *d_siter, double *ttot,
                                  int *status)
{
    static Net::Data data;
    Net::setup_bins(&data);
    const int nbins = Net::NT_LEN - 1;
    std::vector<double2> pairs((size_t)nbins * NT);
    for (int b = 0; b < nbins; b++)
        for (int k = 0; k < NT; k++)
            pairs[(size_t)b * NT + k] = make_double2(tables[k][b], tables[k][b + 1] - tables[k][b]);
    dg::TableSet ts{pairs.data(), nbins, log(data.bounds[0]), data.dbin, data.idbin,
                    data.bounds[0], data.bounds[1], z, {}};
    constexpr int RL = dg::rec_len<NN>();
    std::vector<double> rec((size_t)dims * RL), dbuf((size_t)dims * (NN + 1));
    dg::LockStrip L{*dt, 0.0, 0, 0, 0, 0};
    dg::LockIO io{input, atol, rtol, dims, 1024, dtf, &L, rec.data(), dbuf.data(), 0, dump};
    const dg::KernelCfg kc{10, 50000, 1e-15, 1e-25, 0, 0, nullptr, nullptr, 0};
    const int threads = ((dims + 31) / 32) * 32;
    int nd = 0;
    for (int launch = 0;; launch++) {
        io.resume = launch > 0;
        blockIdx.x = 0;
        gridDim.x = 1;
        blockDim.x = threads;
        hx_setup(threads);
        std::vector<std::thread> lanes;
        for (int t = 0; t < threads; t++)
            lanes.emplace_back([=]() {
                threadIdx.x = t;
                dg::evolve_lockstep_kernel<Net>(io, ts, kc);
            });
        for (auto &th : lanes) th.join();
        if (!dump) break;
        if (L.dumped && nd < max_dumps) {
            for (int c = 0; c < dims; c++) {
                for (int i = 0; i < NN; i++)
                    d_species[((size_t)nd * dims + c) * NN + i] = dbuf[(size_t)c * (NN + 1) + i];
                d_T[(size_t)nd * dims + c] = dbuf[(size_t)c * (NN + 1) + NN];
            }
            d_time[nd] = L.ttot;
            d_dt[nd] = L.dt;
            d_siter[nd] = L.siter;
            nd++;
        }
        if (L.done) break;
    }
    *ttot = L.ttot;
    *dt = L.dt;
    *status = L.status;
    return nd;
}
'''

DRIVER = r'''
/* z_values of dg_api.cuh (cut from its source) */
template <class Net>
struct hx_z {
    using Data = typename Net::Data;
    static constexpr int NT = Net::NT;
%(z_values)s
};
using Net = dgnet_%(name)s::Net;
constexpr int NN = Net::N;
constexpr int NT = Net::NT;
%(launch)s

static void launch(bool mixed, dg::CellIO io, dg::TableSet ts, dg::KernelCfg cfg,
                   unsigned long long *queue)
{
    if (mixed) launch<true>(io, ts, cfg, queue);
    else launch<false>(io, ts, cfg, queue);
}

/* One solve of ncells cells (AoS, mass densities + ge), rtol = rtol_scalar,
 * per-cell dtf, tables in the solver's order; the redistribution's three
 * launches when sweep_budget > 0 (as solve_redistributed in dg_api.cuh);
 * cons_tol: the mixed solve's conservation check (0 off; negative: every
 * converged cell fails it, so every one is re-solved with FP64 solves). */
extern "C" int hx_evolve(double *state, double *atol, const double *dtf, long long ncells,
                         double rtol_scalar, double z, int mixed, int schedule_queue,
                         int sweep_budget, int max_sweeps, const double *const *tables,
                         int *status, int *substeps, int *sweeps, int *failures, double *ttot,
                         double *dt, double cons_tol)
{
    static Net::Data data;
    Net::setup_bins(&data);
    const int nbins = Net::NT_LEN - 1;
    std::vector<double2> pairs((size_t)nbins * NT);
    for (int k = 0; k < NT; k++) {
        double *dst = Net::host_table(&data, k);
        const int len = Net::zdep(k) ? Net::NZ_LEN : Net::NT_LEN;
        for (int b = 0; b < len; b++) dst[b] = tables[k][b];
        if (Net::zdep(k)) continue;
        for (int b = 0; b < nbins; b++)
            pairs[(size_t)b * NT + k] = make_double2(tables[k][b], tables[k][b + 1] - tables[k][b]);
    }
    /* the redshift tables' values at z, as the library computes them on the
     * host before a launch */
    std::vector<double> zvals(NT, 0.0), dzvals(NT, 0.0);
    hx_z<Net>::z_values(&data, z, zvals.data(), dzvals.data());
    dg::TableSet ts{pairs.data(), nbins, log(data.bounds[0]), data.dbin, data.idbin,
                    data.bounds[0], data.bounds[1], z, {}};
    for (int k = 0; k < NT && k < DG_MAX_TABLES; k++) ts.zvals[k] = zvals[k];
    dg::CellIO io{state, atol, nullptr, rtol_scalar, dtf, 0.0, dt, ttot, status, substeps, sweeps,
                  failures, nullptr, NN, 1, ncells};
    /* mixed = 2: the Newton matrix in extended-range FP32 */
    dg::KernelCfg kc{max_sweeps, 50000, 1e-15, 1e-25, 0, 0, nullptr, nullptr, 1, cons_tol,
                     mixed == 2 ? 1 : 0};
    unsigned long long queue = 0;
    unsigned long long *q = schedule_queue ? &queue : nullptr;
    if (sweep_budget <= 0) {
        launch(mixed, io, ts, kc, q);
        return 0;
    }
    std::vector<double> rec((size_t)dg::rec_len<NN>() * ncells);
    kc.sweep_budget = sweep_budget;
    kc.rec = rec.data();
    launch(mixed, io, ts, kc, q);
    const int budgets[2] = {sweep_budget < (1 << 26) ? sweep_budget * 16 : 0, 0};
    int resumed = 0;
    for (int r = 0; r < 2; r++) {
        std::vector<int> list;
        for (long long c = 0; c < ncells; c++)
            if (status[c] == dg::ST_SUSPENDED) list.push_back((int)c);
        const unsigned int count = (unsigned int)list.size();
        resumed += (int)count;
        list.resize((size_t)ncells, -1);
        dg::CellIO io2 = io;
        io2.order = list.data();
        dg::KernelCfg k2 = kc;
        k2.resume = 1;
        k2.resume_count = &count;
        k2.sweep_budget = budgets[r];
        queue = 0;
        launch(mixed, io2, ts, k2, &queue);
    }
    return resumed;
}
'''


def _cut_z_values():
    with open(os.path.join(CSRC, "dg_api.cuh")) as f:
        src = f.read()
    m = re.search(r"^    static void z_values\(.*?^    \}$", src, re.S | re.M)
    assert m, "no z_values in dg_api.cuh"
    return m.group(0)


def _cut_net(name):
    from dengo_gb300.build import network_dir
    with open(os.path.join(network_dir(name), "%s_solver.cu" % name)) as f:
        src = f.read()
    m = re.search(r"^struct Net \{.*?^\};$", src, re.S | re.M)
    assert m, "no Net struct in the generated source of %s" % name
    return "namespace dgnet_%s {\n%s\n}\n" % (name, m.group(0))


def build(name, out_dir, strict=True, engine="lane"):
    """Compile the host engine (``engine`` "lane", "split" or "wide") for network
    ``name`` into ``out_dir``; returns the ctypes library."""
    lib = C.CDLL(compile_engine(name, out_dir, strict, engine))
    return _bind(lib)


def compile_engine(name, out_dir, strict=True, engine="lane"):
    from dengo_gb300.build import network_dir
    tag = "%s_%s%s" % (name, engine, "" if strict else "_lenient")
    src = os.path.join(str(out_dir), "hx_%s.cpp" % tag)
    if engine in ("split", "strip", "wide"):
        # The kernel's block-shared scalars and arrays (``__shared__ int
        # s_any;``) become statics: one CTA runs at a time, and its lanes are
        # threads that must see one copy.  (The dynamic array is dg::dg_smem
        # above.)  The wide engine comes with the split engine, which makes
        # the first launch.
        kernel_source = ""
        for part in (["split", "wide"] if engine == "wide" else [engine]):
            with open(os.path.join(CSRC, "dg_%s.cuh" % part)) as f:
                kernel_source += re.sub(r"(?<!extern )__shared__ ", "static ", f.read())
        prelude = PRELUDE_SPLIT.replace("%(kernel_source)s", kernel_source)
        launch = DRIVER_WIDE_LAUNCH if engine == "wide" else DRIVER_SPLIT_LAUNCH
        driver = (DRIVER_STRIP % dict(name=name) if engine == "strip" else
                  DRIVER % dict(name=name, launch=launch, z_values=_cut_z_values()))
    else:
        prelude, driver = PRELUDE, DRIVER % dict(name=name, launch=DRIVER_LANE_LAUNCH,
                                                 z_values=_cut_z_values())
    with open(src, "w") as f:
        f.write(prelude + '#include "%s_solver.h"\n' % name + _cut_net(name) + driver)
    so = os.path.join(str(out_dir), "hx_%s.so" % tag)
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                           "-w", "-pthread", "-DDG_MIXED_STRICT=%d" % int(strict),
                           "-I", CUDA_INCLUDE, "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                           "-I", network_dir(name), src, "-o", so])
    return so


def _bind(lib):
    lib.hx_evolve.restype = C.c_int
    lib.hx_evolve.argtypes = [P_D, P_D, P_D, C.c_longlong, C.c_double, C.c_double, C.c_int,
                              C.c_int, C.c_int, C.c_int, C.POINTER(P_D), P_I, P_I, P_I, P_I,
                              P_D, P_D, C.c_double]
    return lib


def evolve(lib, tables, state, dtf, z=-1.0, mixed=False, queue=True, sweep_budget=0,
           max_sweeps=10, rtol=1e-6, cons_tol=0.0):
    """Solve ``state`` (cells x N, mass densities + ge) for ``dtf`` with
    atol = 1e-6 x state; returns a dict like ``Solver.solve_host``.
    ``cons_tol``: the mixed solve's conservation check (see hx_evolve)."""
    import numpy as np
    st = np.ascontiguousarray(state, np.float64).copy()
    at = st * 1e-6
    n = st.shape[0]
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(dtf, np.float64), (n,)))
    out = dict(state=st, atol=at, status=np.zeros(n, np.int32), substeps=np.zeros(n, np.int32),
               sweeps=np.zeros(n, np.int32), failures=np.zeros(n, np.int32),
               ttot=np.zeros(n), dt=np.full(n, -1.0))
    tabs = [np.ascontiguousarray(t, np.float64) for t in tables]
    tp = (P_D * len(tabs))(*[t.ctypes.data_as(P_D) for t in tabs])
    ip = lambda a: a.ctypes.data_as(P_I)
    out["resumed"] = lib.hx_evolve(
        st.ctypes.data_as(P_D), at.ctypes.data_as(P_D), d.ctypes.data_as(P_D), n, rtol, z,
        int(mixed), int(queue), int(sweep_budget), int(max_sweeps), tp, ip(out["status"]),
        ip(out["substeps"]), ip(out["sweeps"]), ip(out["failures"]),
        out["ttot"].ctypes.data_as(P_D), out["dt"].ctypes.data_as(P_D), float(cons_tol))
    return out


def evolve_in_subprocess(so, tables, state, dtf, timeout=600, **kw):
    """``evolve`` with the library at path ``so``, run in a child process
    that is killed after ``timeout`` seconds (a host build of a kernel that
    waits on a barrier forever must not hang the test run)."""
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        inp, out = os.path.join(d, "in.npz"), os.path.join(d, "out.npz")
        np.savez(inp, state=state, dtf=np.broadcast_to(np.asarray(dtf, np.float64),
                                                       (len(state),)),
                 **{"table%d" % k: t for k, t in enumerate(tables)})
        code = ("import sys, json, ctypes, numpy as np; sys.path.insert(0, %r); "
                "import host_engine as he; a = np.load(%r); "
                "tabs = [a['table%%d' %% k] for k in range(%d)]; "
                "r = he.evolve(he._bind(ctypes.CDLL(%r)), tabs, a['state'], a['dtf'], **%r); "
                "np.savez(%r, **r)" % (os.path.dirname(os.path.abspath(__file__)), inp,
                                       len(tables), so, kw, out))
        subprocess.run([sys.executable, "-c", code], check=True, timeout=timeout)
        with np.load(out) as r:
            return {k: r[k] for k in r.files}


def lockstep_in_subprocess(so, tables, state, dtf, dump=False, max_dumps=4096, z=-1.0,
                           timeout=600):
    """``dengo_evolve_<n>`` in lockstep (evolve_lockstep_kernel) from the host
    build at path ``so`` on one strip (AoS mass densities + ge, at most 1024
    cells), rtol = 1e-6, atol = 1e-6 x state, in a child process killed after
    ``timeout`` seconds.  Returns the final state, atol, ttot, dt, status and
    (``dump``) the intermediate dumps: ``siter``, ``species`` [k][cells][N],
    ``T`` [k][cells], ``time``, ``timestep``."""
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        inp, out = os.path.join(d, "in.npz"), os.path.join(d, "out.npz")
        np.savez(inp, state=state, **{"table%d" % k: t for k, t in enumerate(tables)})
        code = r'''
import ctypes as C, numpy as np
a = np.load(%(inp)r)
tabs = [np.ascontiguousarray(a["table%%d" %% k]) for k in range(%(nt)d)]
P = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)
lib = C.CDLL(%(so)r)
f = lib.hx_evolve_lockstep
f.restype = C.c_int
f.argtypes = [P, P, P, C.c_int, C.c_double, P, C.c_double, C.POINTER(P), C.c_int, C.c_int,
              P, P, P, P, PI, P, PI]
st = np.ascontiguousarray(a["state"], np.float64).copy()
dims, n = st.shape
rt = np.full_like(st, 1e-06)
at = st * 1e-06
m = %(maxd)d if %(dump)d else 1
sp, T = np.zeros((m, dims, n)), np.zeros((m, dims))
tm, ts, si = np.zeros(m), np.zeros(m), np.zeros(m, np.int32)
ttot, dt, status = np.zeros(1), np.array([-1.0]), np.zeros(1, np.int32)
tp = (P * len(tabs))(*[x.ctypes.data_as(P) for x in tabs])
p = lambda x: x.ctypes.data_as(P)
k = f(p(st), p(rt), p(at), dims, %(dtf)r, p(dt), %(z)r, tp, %(dump)d, m, p(sp), p(T), p(tm),
      p(ts), si.ctypes.data_as(PI), p(ttot), status.ctypes.data_as(PI))
np.savez(%(out)r, state=st, atol=at, ttot=ttot[0], dt=dt[0], status=status[0], siter=si[:k],
         species=sp[:k], T=T[:k], time=tm[:k], timestep=ts[:k])
''' % dict(inp=inp, nt=len(tables), so=so, maxd=int(max_dumps), dump=int(dump),
             dtf=float(dtf), z=float(z), out=out)
        subprocess.run([sys.executable, "-c", code], check=True, timeout=timeout)
        with np.load(out) as r:
            return {k: r[k] for k in r.files}


def run_strip_in_subprocess(so, tables, input_number, tf, niter, z=-1.0, timeout=600):
    """``<n>_run_strip`` (the Cython driver's loop, run_strip_kernel) from the
    host build at path ``so`` on one strip of number densities, in a child
    process killed after ``timeout`` seconds.  Returns the final state,
    atol, ttot, dt, iterations and the per-iteration arrays (``traj``
    [niter][cells][N], ``traj_T`` [niter][cells], ``successful``, ``t``,
    ``dt_traj``)."""
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        inp, out = os.path.join(d, "in.npz"), os.path.join(d, "out.npz")
        np.savez(inp, state=input_number, **{"table%d" % k: t for k, t in enumerate(tables)})
        code = r'''
import ctypes as C, numpy as np
a = np.load(%(inp)r)
tabs = [np.ascontiguousarray(a["table%%d" %% k]) for k in range(%(nt)d)]
P = C.POINTER(C.c_double)
lib = C.CDLL(%(so)r)
f = lib.hx_run_strip
f.restype = C.c_int
f.argtypes = [P, P, P, C.c_int, C.c_double, C.c_int, C.c_double, C.POINTER(P), P, P, P, P,
              C.c_void_p, P, P]
st = np.ascontiguousarray(a["state"], np.float64).copy()
dims, n = st.shape
rt = np.full_like(st, 1e-06)
at = st * 1e-06
ttot, dt = np.zeros(1), np.zeros(1)
traj, traj_T = np.zeros((%(niter)d, dims, n)), np.zeros((%(niter)d, dims))
ok, t, dtt = np.zeros(%(niter)d, np.uint8), np.zeros(%(niter)d), np.zeros(%(niter)d)
tp = (P * len(tabs))(*[x.ctypes.data_as(P) for x in tabs])
p = lambda x: x.ctypes.data_as(P)
it = f(p(st), p(rt), p(at), dims, %(tf)r, %(niter)d, %(z)r, tp, p(ttot), p(dt), p(traj),
       p(traj_T), ok.ctypes.data, p(t), p(dtt))
np.savez(%(out)r, state=st, atol=at, ttot=ttot[0], dt=dt[0], iterations=it, traj=traj,
         traj_T=traj_T, successful=ok.astype(bool), t=t, dt_traj=dtt)
''' % dict(inp=inp, nt=len(tables), so=so, niter=int(niter), tf=float(tf), z=float(z), out=out)
        subprocess.run([sys.executable, "-c", code], check=True, timeout=timeout)
        with np.load(out) as r:
            return {k: r[k] for k in r.files}
