"""The generated device code of each network, compiled for the host.

Each shipped network's ``struct Net`` (temperature, RHS rows, Jacobian
entries, as the CUDA engines call them) is cut out of its generated
``<n>_solver.cu`` and compiled with g++ (``-ffp-contract=off``; the CUDA
build uses ``--fmad=false``), with the engine's table interpolation restated
beside it.  On seeded cells its temperature, rates, right-hand sides and
Jacobian are compared with the oracle's calculate_temperature /
interpolate_rates / calculate_rhs / calculate_jacobian (the reference's
expression text and statement order, rates_and_rate_tables.C.template:
309-599), built with a correctly rounded log T like the device's.  This
checks on the CPU what the generated expressions compute -- the rewrites
(shared reciprocals, integer powers, integer sign tests) included -- for
every network, at several redshifts for the one whose terms read z."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P_D = C.POINTER(C.c_double)
HARNESS = r'''
#include <math.h>
#define __device__
#define __host__
#define __forceinline__ inline
#include "dg_math.h"
#include "dg_xf.h"
#include "%(name)s_solver.h"
%(net)s
using Net = dgnet_%(name)s::Net;
constexpr int N = Net::N;
constexpr int NT = Net::NT;

struct Rates {
    const double *v;
    double operator[](int k) const { return v[k]; }
};
struct Put {
    double *J;
    void operator()(int q, int v, double jv) const { J[v * N + q] = jv; }
    void zero(int q, int v) const { J[v * N + q] = 0.0; }
};
struct PutX {
    double *J;
    void operator()(int q, int v, dg::XF jv) const { J[v * N + q] = dg::xf_to_double(jv); }
    void zero(int q, int v) const { J[v * N + q] = 0.0; }
};

/* Per cell (number densities + ge, AoS): T, the interpolated rates, the
 * RHS and the Jacobian (J[var*N + eq]) as the engines compute them, the
 * interpolation restated from dg_engine.cuh's interpolate(). */
extern "C" int dgx_eval(const double *input, long long ncells, const double *const *tables,
                        double Tlo, double Thi, double z, double *T_out, double *R_out,
                        double *f_out, double *J_out, int *ok_out, double *Jx_out)
{
    if (Net::HAS_Z) return -1;
    const int nbins = Net::NT_LEN - 1;
    const double lb = log(Tlo);
    const double dbin = (log(Thi) - log(Tlo)) / nbins;
    const double idbin = 1.0L / dbin;
    for (long long c = 0; c < ncells; c++) {
        double y[N];
        for (int i = 0; i < N; i++) y[i] = input[c * N + i];
        double T, Tge;
        Net::temperature(y, Tlo, Thi, T, Tge);
        const double logT = dg_log(T);
        const int bin = (int)(idbin * (logT - lb));
        const int bc = bin <= 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
        const double t1 = (lb + (bin) * dbin);
        const double t2 = (lb + (bin + 1) * dbin);
        const double Tdef = (logT - t1) / (t2 - t1);
        double *R = R_out + c * NT;
        for (int k = 0; k < NT; k++) R[k] = tables[k][bc] + Tdef * (tables[k][bc + 1] - tables[k][bc]);
        T_out[c] = T;
        double f[N];
        const bool ok = Net::rhs(y, Rates{R}, T, z, f);
        ok_out[c] = ok ? 1 : 0;
        for (int i = 0; i < N; i++) f_out[c * N + i] = ok ? f[i] : 0.0;
        double *J = J_out + c * N * N;
        for (int i = 0; i < N * N; i++) J[i] = 0.0;
        if (ok) Net::jac(y, Rates{R}, Tge, T, z, Put{J});
        /* the mixed solve's extended-range FP32 Jacobian */
        double *Jx = Jx_out + c * N * N;
        for (int i = 0; i < N * N; i++) Jx[i] = 0.0;
        if (ok) Net::jacx(y, Rates{R}, Tge, T, z, PutX{Jx});
    }
    return 0;
}
'''

CASES = [("primordial", -1.0), ("primordial_compton", -1.0), ("primordial_compton", 0.0),
         ("primordial_compton", 3.0), ("primordial_compton", 19.0), ("oxygen", -1.0)]


def _net_struct(name):
    from dengo_gb300.build import network_dir
    with open(os.path.join(network_dir(name), "%s_solver.cu" % name)) as f:
        src = f.read()
    m = re.search(r"^struct Net \{.*?^\};$", src, re.S | re.M)
    assert m, "no Net struct in the generated source of %s" % name
    return "namespace dgnet_%s {\n%s\n}\n" % (name, m.group(0))


_LIBS = {}


def harness(name, tmp_path_factory):
    if name not in _LIBS:
        from dengo_gb300.build import network_dir
        d = tmp_path_factory.mktemp("dgx_%s" % name)
        src = d / "h.cpp"
        src.write_text(HARNESS % dict(name=name, net=_net_struct(name)))
        so = d / "h.so"
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-w",
                               "-I", os.path.join(ROOT, "dengo_gb300", "csrc"),
                               "-I", os.path.join(ROOT, "include"), "-I", network_dir(name),
                               str(src), "-o", str(so)])
        lib = C.CDLL(str(so))
        lib.dgx_eval.argtypes = [P_D, C.c_longlong, C.POINTER(P_D), C.c_double, C.c_double,
                                 C.c_double, P_D, P_D, P_D, P_D, C.POINTER(C.c_int), P_D]
        _LIBS[name] = lib
    return _LIBS[name]


def _cells(name, n=48):
    from dengo_gb300.networks import build_network
    from dengo_gb300.workloads import oxygen_cells, primordial_cells
    if name.startswith("primordial"):
        a, _ = primordial_cells(n // 2, "config1", seed=4242)
        b, _ = primordial_cells(n - n // 2, "config3", seed=4243)
        st = np.concatenate([a, b])
    else:
        st, _ = oxygen_cells(n, seed=4244)
    net = build_network(name)
    weights = [s.weight for s in sorted(net.required_species)]
    names = [s.name for s in sorted(net.required_species)]
    y = st.copy()
    for i, (w, s) in enumerate(zip(weights, names)):
        if s != "ge":      # mass density -> number density (C.template:158-169)
            y[:, i] = st[:, i] / (w * 1.67e-24)
    return np.ascontiguousarray(y), net


@pytest.mark.parametrize("name,z", CASES)
def test_device_expressions_match_oracle(name, z, tmp_path_factory):
    from dengo_gb300.build import network_dir
    from dengo_gb300.tablefile import read_table_file
    from oracle import Oracle
    y, net = _cells(name)
    ncell, N = y.shape
    from dengo_gb300.codegen.spec import network_spec
    orc = Oracle(name, crlog=True)
    t = read_table_file(os.path.join(network_dir(name), "%s_tables.dgt" % name))
    tabs = [np.ascontiguousarray(t[tb.name]) for tb in network_spec(net, name).tables]
    assert len(tabs) == orc.nt
    tptr = (P_D * len(tabs))(*[a.ctypes.data_as(P_D) for a in tabs])

    # the device expressions, compiled for the host
    lib = harness(name, tmp_path_factory)
    T = np.zeros(ncell)
    R = np.zeros((ncell, orc.nt))
    f = np.zeros((ncell, N))
    J = np.zeros((ncell, N * N))
    ok = np.zeros(ncell, np.int32)
    Jx = np.zeros((ncell, N * N))
    Tlo, Thi = float(net.T_bounds[0]), float(net.T_bounds[1])
    assert lib.dgx_eval(y.ctypes.data_as(P_D), ncell, tptr, Tlo, Thi, z, T.ctypes.data_as(P_D),
                        R.ctypes.data_as(P_D), f.ctypes.data_as(P_D), J.ctypes.data_as(P_D),
                        ok.ctypes.data_as(C.POINTER(C.c_int)), Jx.ctypes.data_as(P_D)) == 0
    assert ok.all()

    # the oracle's strip functions (one strip of all cells)
    from oracle import Network
    onet = Network.in_dll(orc.lib, "dgo_%s_network" % name)
    data = onet.alloc_data(tptr)
    try:
        onet.set_z(data, z)
        inp = y.copy()
        f_ref = np.zeros_like(inp)
        assert onet.rhs(inp.ctypes.data_as(P_D), f_ref.ctypes.data_as(P_D), ncell, N, data) == 0
        T_ref = np.ctypeslib.as_array(onet.Ts(data), shape=(ncell,)).copy()
        J_ref = np.zeros((ncell, N * N))
        assert onet.jac(inp.ctypes.data_as(P_D), J_ref.ctypes.data_as(P_D), ncell, N, data) == 0
    finally:
        onet.free_data(data)

    assert np.array_equal(T, T_ref)
    # right-hand sides and Jacobian entries: sums of cancelling terms, so the
    # scale of an entry's rounding is the cell's largest entry; the integer
    # powers are correctly rounded where libm's pow(x, 3) may not be
    fs = np.abs(f_ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(f - f_ref) <= 1e-13 * fs)
    assert np.mean(np.all(f == f_ref, axis=1)) >= 0.9
    js = np.abs(J_ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(J - J_ref) <= 1e-13 * js)
    assert np.mean(np.all(J == J_ref, axis=1)) >= 0.9
    # the extended-range FP32 Jacobian of the mixed solve: FP32 rounding
    # (2^-24 per operation) but no entry lost to FP32's range -- entries
    # made of tables far below 1e-38 keep their value; measured against
    # each entry's own size, floored at 1e-6 of the row's largest entry
    # (below that cancellation dominates and the entry is negligible in
    # the scaled Newton matrix anyway)
    rows = np.abs(J_ref).reshape(ncell, N, N).max(axis=1, keepdims=True)
    floor = np.maximum(np.abs(J_ref).reshape(ncell, N, N), 1e-6 * rows).reshape(ncell, N * N)
    err = np.where(J_ref == 0, np.abs(Jx), np.abs(Jx - J_ref)) / np.where(floor > 0, floor, 1.0)
    assert err.max() <= 1e-4, err.max()
    # (FP64 subnormals convert to zero by design)
    tiny = (np.abs(J_ref) > 1e-300) & (np.abs(J_ref) < 1e-38)
    if tiny.any():
        assert np.all(Jx[tiny] != 0)
