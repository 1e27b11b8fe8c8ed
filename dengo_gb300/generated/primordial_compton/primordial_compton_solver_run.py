"""THIS FILE HAS BEEN AUTO-GENERATED by dengo_gb300.  DO NOT EDIT.

``run_primordial_compton`` and ``main_run_primordial_compton`` of the reference's Cython module
(rates_and_rate_tables_run.pyx.template), over libprimordial_compton_solver.so and
primordial_compton_tables.dgt next to this file (ctypes; every solve runs on the GPU).
"""
import os
import time

from dengo_gb300.runtime import Solver
from dengo_gb300.tablefile import read_table_file

_HERE = os.path.dirname(os.path.abspath(__file__))
_solver = None


def _get():
    global _solver
    if _solver is None:
        tables = read_table_file(os.path.join(_HERE, "primordial_compton_tables.dgt"))
        _solver = Solver("primordial_compton", tables=tables,
                         lib_path=os.path.join(_HERE, "libprimordial_compton_solver.so"))
    return _solver


def run_primordial_compton(ics, tf, niter=10000, intermediate=1, z=-1.0):
    """The Cython driver's loop on one strip; returns ``(rv, rv_t)``."""
    return _get().run(ics, tf, niter=niter, intermediate=intermediate, z=z)


def main_run_primordial_compton():
    t1 = time.time()
    rc = _get().lib.primordial_compton_main(0, None)
    t2 = time.time()
    print("Total elapsed time: %0.3e" % (t2 - t1))
    return rc
