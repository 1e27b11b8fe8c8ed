"""The sum-of-products tables of the generated networks (Net::sop_*: the RHS
rows and Jacobian entries the wide engine evaluates one term and one sum per
lane) against the generated scalar code (Net::rhs, Net::jac) on random
states and rates, compiled for the host: the same bits for every row and
entry, the rest (rhs_rest / jac_rest) included."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import host_engine as he

HARNESS = r'''
#include <math.h>
#include <string.h>
#include <cuda_runtime.h>
#include "dg_math.h"
#include "dg_slots.cuh"
#include "dg_xf.h"
#include "%(name)s_solver.h"
%(net)s
using Net = dgnet_%(name)s::Net;
constexpr int N = Net::N, NT = Net::NT;
struct Store {
    double *J;
    int *set;
    void operator()(int q, int v, double jv) const { J[v * N + q] = jv; set[v * N + q] = 1; }
    void zero(int q, int v) const { set[v * N + q] = 2; }
};
/* rhs and jac by the scalar code and by the tables; returns the number of
 * rows / entries whose bits differ */
extern "C" int check(const double *yin, const double *R, double Tge, double T, double z)
{
    double y[N], f[N], f2[N], J[N * N], J2[N * N];
    int set[N * N] = {0}, set2[N * N] = {0};
    for (int i = 0; i < N; i++) y[i] = yin[i];
    const dg::Slots<1> Rs{const_cast<double *>(R)};
    if (!Net::rhs(y, Rs, T, z, f)) return -1;
    Net::jac(y, Rs, Tge, T, z, Store{J, set});
    /* tables */
    double OPS[Net::SOP_NOPS + NT + N];
    for (int k = 0; k < NT; k++) OPS[k] = R[k];
    for (int i = 0; i < N; i++) OPS[NT + i] = y[i];
    for (int k = 0; k < Net::SOP_NPOW; k++) {
        const double x = y[Net::sop_pow_sp(k)];
        const int n = Net::sop_pow_n(k);
        OPS[NT + N + k] = n == 2 ? dg_ipow<2>(x) : n == 3 ? dg_ipow<3>(x) : n == 4 ? dg_ipow<4>(x)
                        : n == 5 ? dg_ipow<5>(x) : dg_ipow<6>(x);
    }
    for (int k = 0; k < Net::SOP_NLIT; k++) OPS[Net::SOP_LIT0 + k] = Net::sop_lit(k);
    OPS[Net::SOP_ONE] = 1.0;
    const double md = Net::mdensity_of(y), rmd = 1.0 / md;
    double TV[1024];
    for (int t = 0; t < Net::SOP_RT; t++) {
        const int o0 = Net::sop_rterm(t, 0);
        double v = OPS[o0 & 0x7fff];
        for (int g = 1; g < Net::SOP_FMAX; g++) v = v * OPS[Net::sop_rterm(t, g)];
        TV[t] = (o0 & 0x8000) ? -v : v;
    }
    for (int i = 0; i < N; i++) f2[i] = NAN;
    for (int e = 0; e < Net::SOP_RE; e++) {
        int row, t0, t1, post;
        Net::sop_rentry(e, row, t0, t1, post);
        double acc = TV[t0];
        for (int t = t0 + 1; t < t1; t++) acc = acc + TV[t];
        if (post & 1) acc = acc / md;
        f2[row] = acc;
    }
    double fr[N];
    for (int p = 0; p < Net::SOP_RK; p++) {
        bool ok = p == 0 ? Net::rhs_rest<0>(y, Rs, T, z, fr) : p == 1 ? Net::rhs_rest<1>(y, Rs, T, z, fr)
                                                          : Net::rhs_rest<2>(y, Rs, T, z, fr);
        if (!ok) return -2;
        for (int i = 0; i < N; i++)
            if (Net::sop_rpart(i) == p) f2[i] = fr[i];
    }
    int bad = 0;
    for (int i = 0; i < N; i++) bad += memcmp(&f[i], &f2[i], 8) != 0;
    for (int t = 0; t < Net::SOP_JT; t++) {
        const int o0 = Net::sop_jterm(t, 0);
        double v = OPS[o0 & 0x7fff];
        for (int g = 1; g < Net::SOP_FMAX; g++) v = v * OPS[Net::sop_jterm(t, g)];
        TV[t] = (o0 & 0x8000) ? -v : v;
    }
    for (int e = 0; e < N * N; e++) J2[e] = NAN;
    for (int e = 0; e < Net::SOP_JE; e++) {
        int q, v, t0, t1, post;
        Net::sop_jentry(e, q, v, t0, t1, post);
        double acc = TV[t0];
        for (int t = t0 + 1; t < t1; t++) acc = acc + TV[t];
        if (post & 1) acc = dg_div(acc, md, rmd);
        if (post & 2) acc = acc * Tge;
        J2[v * N + q] = acc;
        set2[v * N + q] = 1;
    }
    for (int p = 0; p < Net::SOP_JK; p++) {
        const Store st{J2, set2};
        bool ok = p == 0 ? Net::jac_rest<0>(y, Rs, Tge, T, z, st) : p == 1 ? Net::jac_rest<1>(y, Rs, Tge, T, z, st)
                                                               : Net::jac_rest<2>(y, Rs, Tge, T, z, st);
        if (!ok) return -3;
    }
    const int ge = Net::IGE;
    const double zr = dg_quot(0.0, md), zc = 0.0 * Tge;
    for (int i = 0; i < N; i++) {
        if (!Net::jraw(ge, i)) { J2[i * N + ge] = i == ge ? zr * Tge : zr; set2[i * N + ge] = 1; }
        if (i != ge && !Net::jraw(i, ge)) { J2[ge * N + i] = zc; set2[ge * N + i] = 1; }
    }
    for (int e = 0; e < N * N; e++) {
        const int v = e / N, q = e - v * N;
        if (set[e] == 2) { bad += !(!Net::jraw(q, v) && q != ge && v != ge && set2[e] == 0); continue; }
        bad += set2[e] != 1 || memcmp(&J[e], &J2[e], 8) != 0;
    }
    return bad;
}
'''


@pytest.mark.parametrize("name", ["primordial", "primordial_compton", "oxygen", "oxygen_uvb"])
def test_sop_tables_equal_scalar_code(name, tmp_path):
    from dengo_gb300.build import network_dir
    from dengo_gb300.codegen import render_solver  # noqa: F401 (the generated sources exist)
    src = tmp_path / ("sop_%s.cpp" % name)
    src.write_text(HARNESS % dict(name=name, net=he._cut_net(name)))
    so = tmp_path / ("sop_%s.so" % name)
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-w",
                           "-I", he.CUDA_INCLUDE, "-I", he.CSRC, "-I", os.path.join(he.ROOT, "include"),
                           "-I", network_dir(name), str(src), "-o", str(so)])
    lib = C.CDLL(str(so))
    P = C.POINTER(C.c_double)
    lib.check.argtypes = [P, P, C.c_double, C.c_double, C.c_double]
    lib.check.restype = C.c_int
    rng = np.random.default_rng(7)
    import re
    text = open(os.path.join(network_dir(name), "%s_solver.cu" % name)).read()
    N = int(re.search(r"static constexpr int N = (\d+);", text).group(1))
    NT = int(re.search(r"static constexpr int NT = (\d+);", text).group(1))
    for _ in range(200):
        y = np.exp(rng.uniform(-80, 20, N))
        R = np.exp(rng.uniform(-60, 10, NT)) * rng.choice([-1.0, 1.0], NT)
        r = lib.check(y.ctypes.data_as(P), R.ctypes.data_as(P), float(np.exp(rng.uniform(-5, 5))),
                      float(np.exp(rng.uniform(2, 20))), 1.5)
        assert r == 0, r
