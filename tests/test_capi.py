"""The C-ABI libraries load without a GPU and export every entry point
include/dengo_gb300.h declares (no compute call is made here)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(network):
    text = open(os.path.join(ROOT, "include", "dengo_gb300.h")).read()
    macro = text[text.index("#define DENGO_DECLARE_NETWORK"):]
    macro = macro[:macro.index("/* The unprefixed")]
    names = set(re.findall(r"\b(n##_\w+|\w+_##n|\w+##_##n)\s*\(", macro))
    out = set()
    for nm in names:
        out.add(nm.replace("n##_", network + "_").replace("_##n", "_" + network)
                .replace("##", ""))
    out |= {"ensure_electron_consistency", "temperature_from_mass_density", "BE_chem_solve",
            "dengo_default_config"}
    return out


@pytest.fixture(scope="module")
def libpath():
    from dengo_gb300.build import build_network, library_path
    p = library_path("primordial")
    if not os.path.exists(p):
        build_network("primordial")
    return p


def test_every_declared_symbol_is_exported(libpath):
    want = declared("primordial")
    assert "dengo_evolve_primordial" in want and "primordial_solve_cells_device" in want
    nm = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True,
                        text=True).stdout
    have = {line.split()[-1] for line in nm.splitlines()}
    missing = sorted(want - have)
    assert not missing, missing


def test_library_loads_without_gpu(libpath):
    lib = C.CDLL(libpath)
    lib.primordial_nspecies.restype = C.c_int
    assert lib.primordial_nspecies() == 10
    lib.primordial_ntables.restype = C.c_int
    assert lib.primordial_ntables() == 44
    lib.primordial_species_name.restype = C.c_char_p
    assert lib.primordial_species_name(9) == b"ge"


def test_python_default_config_is_the_library_default(libpath):
    """Solver.default_config() mirrors dengo_default_config() field by field
    (the call needs no GPU)."""
    from dengo_gb300.runtime import Solver, SolverConfig
    lib = C.CDLL(libpath)
    lib.dengo_default_config.argtypes = [C.POINTER(SolverConfig)]
    c = SolverConfig()
    lib.dengo_default_config(C.byref(c))
    py = Solver.default_config()
    for name, _ in SolverConfig._fields_:
        assert getattr(c, name) == getattr(py, name), name
    assert c.warps_per_cell == 4 and c.sweep_budget == 2000


def test_runtime_fails_loudly_without_library(tmp_path):
    from dengo_gb300.runtime import load_library
    with pytest.raises(RuntimeError, match="not built"):
        load_library("primordial", path=str(tmp_path / "missing.so"))


HOST_C = r'''
/* An Enzo-style host code: plain C99 against the generated header, linked
 * with the network library. */
#include <stdio.h>
#include "primordial_solver.h"

int evolve_grid(double dtf, double z, double *fields, double *rtol, double *atol,
                long long ncells)
{
    int nf = 0;
    char **names = NULL;
    primordial_data *data = primordial_setup_data(&nf, &names);
    if (!data) {
        fprintf(stderr, "%s\n", primordial_last_error());
        return -1;
    }
    double dt = -1.0;
    double ttot = dengo_evolve_primordial(dtf, &dt, z, fields, rtol, atol, ncells, data);
    dengo_cell_batch b = {0};
    b.ncells = ncells;
    b.cell_stride = 10;
    b.species_stride = 1;
    b.state = fields;
    b.atol = atol;
    b.rtol_scalar = 1e-6;
    b.dtf_scalar = dtf;
    dengo_solver_config cfg;
    dengo_default_config(&cfg);
    cfg.precision = DENGO_MIXED;
    int rc = primordial_solve_cells_host(data, &b, z, &cfg);
    /* a GPU-resident code passes device pointers and a stream instead */
    rc |= primordial_solve_cells_device(data, &b, z, &cfg, NULL);
    rc |= primordial_solve_cells_device_noalloc(data, &b, z, &cfg, NULL);
    primordial_free_data(data);
    return (ttot < dtf || rc != 0) ? 1 : 0;
}

int main(void) { return 0; }
'''


def test_header_serves_a_c99_host_code(libpath, tmp_path):
    """A C99 program using the reference's entry points and the batch API
    compiles against the generated header and links against the library
    (nothing is run: that needs a GPU)."""
    from dengo_gb300.build import network_dir
    src = tmp_path / "host.c"
    src.write_text(HOST_C)
    exe = tmp_path / "host"
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic",
                           "-I", os.path.join(ROOT, "include"), "-I", network_dir("primordial"),
                           str(src), "-o", str(exe), "-L", os.path.dirname(libpath),
                           "-lprimordial_solver", "-Wl,-rpath," + os.path.dirname(libpath)])
    assert exe.exists()
