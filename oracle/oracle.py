"""ORACLE -- test infrastructure, not part of the product.

Python access to the C restatement (be_oracle.c + gen/<name>_oracle.c) and,
where it was built, to the reference's own solver (oracle/_ref).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
P_D = C.POINTER(C.c_double)
P_I = C.POINTER(C.c_int)
P_L = C.POINTER(C.c_longlong)

CFLAGS = ["-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-w"]


class Config(C.Structure):
    _fields_ = [("max_sweeps", C.c_int), ("max_substeps", C.c_int),
                ("dt_ratio_floor", C.c_double), ("floor_value", C.c_double)]


def build_oracle(name="primordial", force=False, crlog=False):
    """Compile the C restatement for network ``name`` (gcc).  ``crlog``: the
    variant whose log T is correctly rounded instead of libm's."""
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libdgo_%s%s.so" % (name, "_crlog" if crlog else ""))
    srcs = [os.path.join(HERE, "be_oracle.c"), os.path.join(HERE, "gen", "%s_oracle.c" % name)]
    if force or not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out)
                                               for s in srcs):
        extra = ["-DDGO_LOG=dgo_crlog"] if crlog else []
        libs = ["-lquadmath"] if platform.machine() == "x86_64" else []
        subprocess.check_call(["gcc"] + CFLAGS + extra + srcs + ["-o", out, "-lm"] + libs)
    return out


def _dp(a):
    return a.ctypes.data_as(P_D)


_STRIP_F = C.CFUNCTYPE(C.c_int, P_D, P_D, C.c_int, C.c_int, C.c_void_p)


class Network(C.Structure):
    """``dgo_network`` (be_oracle.h): one network's strip functions."""
    _fields_ = [("name", C.c_char_p), ("nchem", C.c_int), ("ige", C.c_int), ("unit", P_D),
                ("input_is_number", C.c_int), ("rhs", _STRIP_F), ("jac", _STRIP_F),
                ("electrons", C.CFUNCTYPE(None, P_D, C.c_int, C.c_int)),
                ("alloc_data", C.CFUNCTYPE(C.c_void_p, C.POINTER(P_D))),
                ("free_data", C.CFUNCTYPE(None, C.c_void_p)),
                ("set_z", C.CFUNCTYPE(None, C.c_void_p, C.c_double)),
                ("Ts", C.CFUNCTYPE(P_D, C.c_void_p))]


class Oracle:
    """The C restatement of the reference solver for one network."""

    def __init__(self, name="primordial", crlog=False):
        self.name = name
        self.lib = C.CDLL(build_oracle(name, crlog=crlog))
        self.net_addr = C.addressof(C.c_char.in_dll(self.lib, "dgo_%s_network" % name))
        self.lib.dgo_default_config.restype = Config
        self.lib.dgo_evolve_cells.argtypes = [
            C.c_void_p, C.POINTER(P_D), P_D, P_D, C.c_double, P_D, P_D, P_D, C.c_longlong,
            C.POINTER(Config), P_D, P_I, P_L, P_L, P_L, C.c_int]
        self.lib.dgo_evolve.argtypes = [C.c_void_p, C.c_void_p, C.c_double, P_D, C.c_double,
                                        P_D, P_D, P_D, C.c_longlong, C.POINTER(Config),
                                        C.c_void_p]
        self.lib.dgo_evolve.restype = C.c_double
        self.nt = getattr(self.lib, "dgo_%s_ntables" % name)()
        ntab = getattr(self.lib, "dgo_%s_table_len" % name)
        ntab.argtypes = [C.c_int]
        self.table_len = [ntab(k) for k in range(self.nt)]
        tname = getattr(self.lib, "dgo_%s_table_name" % name)
        tname.argtypes, tname.restype = [C.c_int], C.c_char_p
        self.table_names = [tname(k).decode() for k in range(self.nt)]

    def tables_from_bundle(self, path):
        """The tables of a ``<name>_tables.dgt`` bundle in this network's
        table order."""
        import sys
        sys.path.insert(0, os.path.dirname(HERE))
        from dengo_gb300.tablefile import read_table_file
        tabs = read_table_file(path)
        return [tabs[k] for k in self.table_names]

    def config(self, max_sweeps=10, max_substeps=50000):
        c = self.lib.dgo_default_config()
        c.max_sweeps, c.max_substeps = max_sweeps, max_substeps
        return c

    def _tables(self, tables_in_order):
        keep = [np.ascontiguousarray(t, np.float64) for t in tables_in_order]
        return keep, (P_D * len(keep))(*[_dp(t) for t in keep])

    def evolve_cells(self, tables_in_order, state, dtf, dt=None, z=-1.0, rtol=None, atol=None,
                     nthreads=0, max_sweeps=10, max_substeps=50000):
        """Per-cell reference semantics (dengo_evolve with dims = 1 per cell).

        state: (cells, N) AoS mass densities + ge.  Returns a dict."""
        st = np.ascontiguousarray(state, np.float64).copy()
        n = st.shape[0]
        rt = np.full_like(st, 1e-6) if rtol is None else np.ascontiguousarray(rtol, np.float64).copy()
        at = (1e-6 * st) if atol is None else np.ascontiguousarray(atol, np.float64).copy()
        dtf = np.broadcast_to(np.asarray(dtf, np.float64), (n,)).copy()
        dt = np.full(n, -1.0) if dt is None else np.broadcast_to(np.asarray(dt, np.float64), (n,)).copy()
        keep, tp = self._tables(tables_in_order)
        ttot = np.zeros(n)
        status = np.zeros(n, np.int32)
        sub, sw, fl = (np.zeros(n, np.int64) for _ in range(3))
        cfg = self.config(max_sweeps, max_substeps)
        self.lib.dgo_evolve_cells(self.net_addr, tp, _dp(dtf), _dp(dt), float(z), _dp(st),
                                  _dp(rt), _dp(at), n, C.byref(cfg), _dp(ttot),
                                  status.ctypes.data_as(P_I), sub.ctypes.data_as(P_L),
                                  sw.ctypes.data_as(P_L), fl.ctypes.data_as(P_L), int(nthreads))
        return dict(state=st, atol=at, dt=dt, ttot=ttot, status=status, substeps=sub,
                    sweeps=sw, failures=fl)


class Stats(C.Structure):
    _fields_ = [("substeps_ok", C.c_longlong), ("substeps_fail", C.c_longlong),
                ("sweeps", C.c_longlong), ("status", C.c_int)]


_HOOK_F = C.CFUNCTYPE(None, C.c_void_p, C.c_int, P_D, P_D, C.c_longlong, C.c_int, C.c_double,
                      C.c_double)


def evolve_strip(orc, tables_in_order, state, dtf, z=-1.0, dt=-1.0, intermediate=False,
                 rtol=None, atol=None, max_substeps=50000):
    """dengo_evolve_<name> over one strip in lockstep (dims = the number of
    cells; the reference's own semantics for dims > 1): one dt and one
    Newton loop for the whole strip.  Returns a dict; with ``intermediate``
    also ``intermediate``: one dict per accepted substep holding what the
    reference writes to <name>_intermediate_%06d (siter, species = prev,
    T, time, timestep)."""
    st = np.ascontiguousarray(state, np.float64).copy()
    rt = np.full_like(st, 1e-6) if rtol is None else np.ascontiguousarray(rtol, np.float64).copy()
    at = (1e-6 * st) if atol is None else np.ascontiguousarray(atol, np.float64).copy()
    keep, tp = orc._tables(tables_in_order)
    net = Network.in_dll(orc.lib, "dgo_%s_network" % orc.name)
    data = net.alloc_data(tp)
    dumps = []

    def hook(ctx, siter, prev, Ts, dims, nchem, ttot, dt_next):
        dumps.append(dict(siter=siter,
                          species=np.ctypeslib.as_array(prev, (dims, nchem)).copy(),
                          T=np.ctypeslib.as_array(Ts, (dims,)).copy(),
                          time=ttot, timestep=dt_next))

    cb = _HOOK_F(hook)
    orc.lib.dgo_set_intermediate_hook.argtypes = [_HOOK_F, C.c_void_p]
    if intermediate:
        orc.lib.dgo_set_intermediate_hook(cb, None)
    try:
        d = C.c_double(dt)
        cfg = orc.config(max_substeps=max_substeps)
        ttot = orc.lib.dgo_evolve(orc.net_addr, data, float(dtf), C.byref(d), float(z), _dp(st),
                                  _dp(rt), _dp(at), st.shape[0], C.byref(cfg), None)
    finally:
        if intermediate:
            orc.lib.dgo_set_intermediate_hook(_HOOK_F(), None)
        net.free_data(data)
    out = dict(state=st, atol=at, ttot=ttot, dt=d.value)
    if intermediate:
        out["intermediate"] = dumps
    return out


def run_strip(orc, tables_in_order, input_number, tf, niter, z=-1.0, trajectories=False):
    """The Cython driver's loop (dgo_run_strip_traj) on one strip of number
    densities (already divided by the weights).  Returns a dict; with
    ``trajectories`` also the driver's intermediate arrays: ``traj``
    (niter, cells, N), ``traj_T`` (niter, cells), ``successful``, ``t``,
    ``dt`` (niter), zeros after the last iteration taken."""
    inp = np.ascontiguousarray(input_number, np.float64).copy()
    dims, n = inp.shape
    rt = np.full_like(inp, 1e-06)
    at = inp * 1e-06
    keep, tp = orc._tables(tables_in_order)
    ttot, dt, st = C.c_double(), C.c_double(), Stats()
    cfg = orc.config()
    fn = orc.lib.dgo_run_strip_tables
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(P_D), C.c_double, C.c_int, C.c_double, P_D, P_D, P_D,
                   C.c_int, C.POINTER(Config), C.POINTER(C.c_double), C.POINTER(C.c_double),
                   C.POINTER(Stats), P_D, P_D, C.c_void_p, P_D, P_D]
    tr = dict(traj=np.zeros((niter, dims, n)), traj_T=np.zeros((niter, dims)),
              successful=np.zeros(niter, np.uint8), t=np.zeros(niter),
              dt=np.zeros(niter)) if trajectories else None
    args = ([_dp(tr["traj"]), _dp(tr["traj_T"]), tr["successful"].ctypes.data, _dp(tr["t"]),
             _dp(tr["dt"])] if tr else [None] * 5)
    it = fn(orc.net_addr, tp, float(tf), int(niter), float(z), _dp(inp), _dp(rt), _dp(at),
            dims, C.byref(cfg), C.byref(ttot), C.byref(dt), C.byref(st), *args)
    out = dict(state=inp, atol=at, ttot=ttot.value, dt=dt.value, iterations=it,
               substeps_ok=st.substeps_ok, substeps_fail=st.substeps_fail, sweeps=st.sweeps)
    if tr:
        tr["successful"] = tr["successful"].astype(bool)
        out["trajectories"] = tr
    return out


class Reference:
    """The reference's own generated solver, built by oracle/ref_build.py
    (only where the reference checkout exists)."""

    def __init__(self, name="primordial", intermediate=False):
        tag = name + ("_intermediate" if intermediate else "")
        path = os.path.join(REF, "libref_%s.so" % tag)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        # the tables, and (intermediate build) its intermediate files, live here
        os.environ["DGO_REF_TABLE_DIR"] = os.path.join(REF, tag)
        self.lib = C.CDLL(path)
        self.lib.ref_evolve_cells.argtypes = [P_D, P_D, C.c_double, P_D, P_D, P_D, C.c_longlong,
                                              P_D, C.c_int]
        self.lib.ref_setup.restype = C.c_void_p
        self.lib.ref_rs.restype = P_D
        self.lib.ref_rs.argtypes = [C.c_void_p, C.c_int]
        self.lib.ref_Ts.restype = P_D
        self.lib.ref_Ts.argtypes = [C.c_void_p]
        self.lib.ref_dTs_ge.restype = P_D
        self.lib.ref_dTs_ge.argtypes = [C.c_void_p]
        for f in ("ref_rhs", "ref_jac"):
            getattr(self.lib, f).argtypes = [P_D, P_D, C.c_int, C.c_int, C.c_void_p]
        self.lib.ref_temperature.argtypes = [C.c_void_p, P_D, C.c_int, C.c_int]
        self.lib.ref_interpolate.argtypes = [C.c_void_p, C.c_int]
        self.lib.ref_electrons.argtypes = [P_D, C.c_int, C.c_int]
        self.lib.ref_evolve.argtypes = [C.c_void_p, C.c_double, P_D, C.c_double, P_D, P_D, P_D,
                                        C.c_longlong]
        self.lib.ref_evolve.restype = C.c_double
        self.lib.ref_BE_chem_solve.argtypes = [P_D, C.c_double, P_D, P_D, C.c_int, C.c_int, P_D,
                                               C.c_void_p, P_D, P_D, P_D, P_D]
        self.N = self.lib.ref_nchem()

    def evolve_cells(self, state, dtf, dt=None, z=-1.0, rtol=None, atol=None, nthreads=0):
        st = np.ascontiguousarray(state, np.float64).copy()
        n = st.shape[0]
        rt = np.full_like(st, 1e-6) if rtol is None else np.ascontiguousarray(rtol, np.float64).copy()
        at = (1e-6 * st) if atol is None else np.ascontiguousarray(atol, np.float64).copy()
        dtf = np.broadcast_to(np.asarray(dtf, np.float64), (n,)).copy()
        dt = np.full(n, -1.0) if dt is None else np.broadcast_to(np.asarray(dt, np.float64), (n,)).copy()
        ttot = np.zeros(n)
        self.lib.ref_evolve_cells(_dp(dtf), _dp(dt), float(z), _dp(st), _dp(rt), _dp(at), n,
                                  _dp(ttot), int(nthreads))
        return dict(state=st, atol=at, dt=dt, ttot=ttot)
