"""ORACLE -- test infrastructure.  Builds the reference's own solver into
``oracle/_ref/`` so the C restatement can be pinned against it.

Recipe (runs only where the reference checkout exists):

1. Import the reference package read-only from ``REF_ROOT`` (below) with
   compatibility shims that change no arithmetic:
   * ``h5py`` is replaced by a writer of raw float64 files (the container has
     no HDF5); ``docutils.utils.roman`` (imported, unused) is stubbed;
   * the cooling equations' pre-rename species names (``HI``, ``HeII``, ...)
     are aliased to the registered species (dengo/primordial_cooling.py vs
     dengo/primordial_rates.py:36-43);
   * ``CoolingAction.species`` concatenates lists instead of dict views
     (reaction_classes.py:356, a Python-2 idiom);
   * ``CoolingAction`` is given an order by name so ``write_solver`` can sort
     it (chemical_network.py:314);
   * temporaries are parsed with the species and table symbols in scope, so
     ``galdl`` of ``gloverabel08`` refers to the species symbols
     (reaction_classes.py:346-350) and ``comp`` of ``compton`` to its table
     rather than to ``sympy.comp`` (primordial_cooling.py:280-292).
2. Build the primordial network (all reactions; all cooling actions except
   ``compton``, or all of them for ``primordial_compton``; 1024 bins over
   1-1e9 K), or an ion-by-ion network, and call the reference's
   ``write_solver(..., ode_solver_source=None)`` into ``oracle/_ref/<name>/``:
   the rendered ``<name>_solver.C/.h`` and the tables.
3. Compile the rendered solver together with the reference's
   ``dengo/solvers/BE_chem_solve.C`` (read where it lies), a small C harness
   written here, and the header-only HDF5 stand-in in ``oracle/hdf5_shim/``:
   ``g++ -O2 -ffp-contract=off -fopenmp -shared``.

Output: ``oracle/_ref/libref_<name>.so`` exporting ``ref_*`` functions.

``build_cython_driver(name)`` also compiles the reference's Cython driver
as its ``write_solver`` rendered it (``<name>_solver_run.pyx``, from
rates_and_rate_tables_run.pyx.template): Cython with ``language_level=2``
(the template is Python-2 code) in C++ mode, linked with the rendered solver
and ``BE_chem_solve.C`` into ``oracle/_ref/<name>/<name>_solver_run<ext>``,
importable as the reference's own ``run_<name>``.
"""

import os
import subprocess
import sys
import sysconfig
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $DGO_REFERENCE_ROOT, else a "reference" directory
# beside this repository's root.
REF_ROOT = os.environ.get(
    "DGO_REFERENCE_ROOT",
    os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                 "reference"))
OUT = os.path.join(HERE, "_ref")

ALIASES = dict(HI="H_1", HII="H_2", HM="H_m0", HeI="He_1", HeII="He_2",
               HeIII="He_3", H2I="H2_1", H2II="H2_2")


def _install_shims():
    h5 = types.ModuleType("h5py")

    class _Reader:
        """The UV-background input files (input/photoionization/<el>_ion_by_
        ion_photoionization_<bg>.h5, input/photoheating/...), served from the
        seeded stand-in tables of dengo_gb300/ion_by_ion.py."""

        def __init__(self, path):
            base = os.path.basename(path)
            self.element = base.split("_")[0]
            self.kind = "photoionization" if "photoionization" in base else "photoheating"

        def __getitem__(self, key):
            from dengo_gb300.ion_by_ion import photo_data
            z, vals = photo_data(self.element, key if key != "z" else self.element + "_1",
                                 self.kind)
            return z if key == "z" else vals

        def close(self):
            pass

    class _File:
        def __new__(cls, path, mode="r"):
            if path.startswith("input/photo"):
                return _Reader(path)
            return super().__new__(cls)

        def __init__(self, path, mode="r"):
            self.path = path
            os.makedirs(path + ".d", exist_ok=True)

        def create_dataset(self, name, data):
            np.ascontiguousarray(data, dtype="<f8").tofile(
                os.path.join(self.path + ".d", name.strip("/") + ".f64"))

        def close(self):
            pass

    h5.File = _File
    sys.modules["h5py"] = h5
    du = types.ModuleType("docutils")
    duu = types.ModuleType("docutils.utils")
    dur = types.ModuleType("docutils.utils.roman")
    du.utils, duu.roman = duu, dur
    sys.modules.update({"docutils": du, "docutils.utils": duu,
                        "docutils.utils.roman": dur})


def _reference_primordial(with_compton=False):
    sys.path.insert(0, REF_ROOT)
    _install_shims()
    import sympy
    import dengo.reaction_classes as rc
    import dengo.chemical_network as cn
    from dengo.primordial_rates import setup_primordial
    setup_primordial()
    for a, n in ALIASES.items():
        rc.species_registry[a] = rc.species_registry[n]

    def equation(self):
        if self._eq is not None:
            return self._eq
        symbols = {n: s.symbol for n, s in rc.species_registry.items()}
        ta = {n: sympy.Symbol("%s_%s[i]" % (self.name, n)) for n in self.tables}
        tp = {n: sympy.Symbol(n) for n in self.temporaries}
        self.table_symbols.update(ta)
        self.temp_symbols.update(tp)
        symbols.update(ta)
        symbols.update(tp)
        self._eq = eval(self._equation, symbols)
        for n, e in self.temporaries.items():
            scope = {k: s.symbol for k, s in rc.species_registry.items()}
            scope.update(ta)
            self._eq = self._eq.subs(n, sympy.sympify(e, locals=scope))
        return self._eq

    def species(self):
        self.equation
        bad = set(list(self.temp_symbols.values()) + list(self.table_symbols.values()))
        return {rc.species_registry[str(s).replace("[i]", "")]
                for s in self.equation.atoms(sympy.Symbol) if s not in bad}

    rc.CoolingAction.equation = property(equation)
    rc.CoolingAction.species = property(species)
    rc.CoolingAction.__lt__ = lambda a, b: a.name < b.name
    import dengo.primordial_cooling  # noqa: F401
    net = cn.ChemicalNetwork()
    for c in sorted(rc.cooling_registry):
        if c != "compton" or with_compton:
            net.add_cooling(c)
    for r in sorted(rc.reaction_registry):
        net.add_reaction(r)
    net.init_temperature((1e0, 1e9), n_bins=1024)
    return net


def _reference_oxygen(photo_background=None):
    """The reference's own ion-by-ion setup (dengo/ion_by_ion.py:33-56) for
    H, O and He.  ChiantiPy is absent: a stand-in module lets
    ``chianti_rate`` register its reactions (it only checks that ChiantiPy
    imported), and every rate and cooling table is then replaced by the
    seeded synthetic curve this package tabulates for the same ion
    (dengo_gb300/ion_by_ion.py), so both sides consume identical tables.  The
    reference's Python-2 implicit import of ``reaction_classes``
    (ion_by_ion.py:24) is satisfied by aliasing the module."""
    sys.path.insert(0, REF_ROOT)
    sys.path.insert(0, os.path.dirname(HERE))
    _install_shims()
    import sympy
    import dengo.reaction_classes as rc
    import dengo.chemical_network as cn
    sys.modules["reaction_classes"] = rc
    rc.ch = types.ModuleType("chianti_stand_in")
    rc.chu = rc.ch
    _patch_cooling_actions(rc, sympy)
    from dengo.ion_by_ion import setup_ionization
    from dengo_gb300 import ion_by_ion as mine
    net = cn.ChemicalNetwork()
    net.add_species("de")
    for atom in ("H", "O", "He"):
        s, c, r = setup_ionization(atom, photo_background=photo_background)
        num = {"H": 1, "He": 2, "O": 8}[atom]
        for i in range(num + 1):
            name = rc.species_registry["%s_%d" % (atom, i + 1)].name
            if "%s_i" % name in rc.reaction_registry:
                rc.reaction_registry["%s_i" % name].coeff_fn = mine.ionization_rate(atom, i)
            if "%s_r" % name in rc.reaction_registry:
                rc.reaction_registry["%s_r" % name].coeff_fn = mine.recombination_rate(atom, i)
            act = rc.cooling_registry["%s_c" % name]
            act.tables["%s_c" % name] = mine.cooling_rate(atom, i)
        net.add_collection(s, c, r)
    net.init_temperature((1e0, 1e10), n_bins=8192)
    if photo_background is not None:
        net.init_redshift((0.0, 15.0), n_z_bins=100)
    return net


def _patch_cooling_actions(rc, sympy):
    def equation(self):
        if self._eq is not None:
            return self._eq
        symbols = {n: s.symbol for n, s in rc.species_registry.items()}
        ta = {n: sympy.Symbol("%s_%s[i]" % (self.name, n)) for n in self.tables}
        tp = {n: sympy.Symbol(n) for n in self.temporaries}
        self.table_symbols.update(ta)
        self.temp_symbols.update(tp)
        symbols.update(ta)
        symbols.update(tp)
        self._eq = eval(self._equation, symbols)
        for n, e in self.temporaries.items():
            scope = {k: s.symbol for k, s in rc.species_registry.items()}
            scope.update(ta)
            self._eq = self._eq.subs(n, sympy.sympify(e, locals=scope))
        return self._eq

    def species(self):
        self.equation
        bad = set(list(self.temp_symbols.values()) + list(self.table_symbols.values()))
        return {rc.species_registry[str(s).replace("[i]", "")]
                for s in self.equation.atoms(sympy.Symbol) if s not in bad}

    rc.CoolingAction.equation = property(equation)
    rc.CoolingAction.species = property(species)
    rc.CoolingAction.__lt__ = lambda a, b: a.name < b.name


HARNESS = r"""
/* ORACLE -- test infrastructure: C entry points over the reference's
 * rendered solver, written by oracle/ref_build.py. */
#include "%(n)s_solver.h"
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif
void %(n)s_calculate_temperature(%(n)s_data *, double *, int, int);
void %(n)s_interpolate_rates(%(n)s_data *, int);
static const size_t dgo_rs_off[] = { %(rs)s };
extern "C" {
void *ref_setup(void) { return %(n)s_setup_data(NULL, NULL); }
void ref_free(void *d) { free(d); }
int ref_nchem(void) { return NSPECIES; }
double ref_evolve(void *d, double dtf, double *dt, double z, double *input,
                  double *rtol, double *atol, long long dims)
{ return dengo_evolve_%(n)s(dtf, *dt, z, input, rtol, atol, dims, (%(n)s_data *)d); }
int ref_rhs(double *in, double *out, int ns, int nc, void *d)
{ return calculate_rhs_%(n)s(in, out, ns, nc, d); }
int ref_jac(double *in, double *out, int ns, int nc, void *d)
{ return calculate_jacobian_%(n)s(in, out, ns, nc, d); }
void ref_temperature(void *d, double *in, int ns, int nc)
{ %(n)s_calculate_temperature((%(n)s_data *)d, in, ns, nc); }
void ref_interpolate(void *d, int ns) { %(n)s_interpolate_rates((%(n)s_data *)d, ns); }
const double *ref_Ts(void *d) { return ((%(n)s_data *)d)->Ts; }
const double *ref_dTs_ge(void *d) { return ((%(n)s_data *)d)->dTs_ge; }
void ref_electrons(double *in, int ns, int nc) { ensure_electron_consistency(in, ns, nc); }
int ref_BE_chem_solve(double *u, double dt, double *rtol, double *atol, int ns, int nc,
                      double *scaling, void *d, double *u0, double *s, double *gu, double *Ju)
{ return BE_chem_solve(calculate_rhs_%(n)s, calculate_jacobian_%(n)s, u, dt, rtol, atol,
                       ns, nc, scaling, d, u0, s, gu, Ju); }
const double *ref_rs(void *d, int k) {
    return (const double *)((const char *)d + dgo_rs_off[k]);
}
void ref_evolve_cells(const double *dtf, double *dt, double z, double *input, double *rtol,
                      double *atol, long long ncells, double *ttot, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        %(n)s_data *d = %(n)s_setup_data(NULL, NULL);
        long long c;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (c = 0; c < ncells; c++) {
            double t = dt[c];
            ttot[c] = dengo_evolve_%(n)s(dtf[c], t, z, input + c * NSPECIES,
                                         rtol + c * NSPECIES, atol + c * NSPECIES, 1, d);
            dt[c] = t;
        }
        free(d);
    }
}
}
"""


def build(name="primordial", intermediate=False):
    """Render and compile one network in a fresh interpreter (the reference's
    registries are module globals, so networks are built one per process).
    ``intermediate``: render it with ``write_intermediate_solutions`` set, so
    that its dengo_evolve writes <name>_intermediate_%06d files (the
    library is libref_<name>_intermediate.so)."""
    if name not in ("primordial", "primordial_compton", "oxygen", "oxygen_uvb"):
        raise ValueError("networks rendered with the reference here: primordial, "
                         "primordial_compton, oxygen, oxygen_uvb")
    if not os.path.isdir(os.path.join(REF_ROOT, "dengo")):
        raise FileNotFoundError("reference checkout not found at %s" % REF_ROOT)
    tag = name + ("_intermediate" if intermediate else "")
    if "dengo" in sys.modules:
        lib = os.path.join(OUT, "libref_%s.so" % tag)
        subprocess.check_call([sys.executable, os.path.abspath(__file__), name] +
                              (["intermediate"] if intermediate else []))
        return lib
    if name.startswith("primordial"):
        net = _reference_primordial(with_compton=(name == "primordial_compton"))
    else:
        net = _reference_oxygen("HM12" if name == "oxygen_uvb" else None)
    net.write_intermediate_solutions = bool(intermediate)
    odir = os.path.join(OUT, tag)
    os.makedirs(odir, exist_ok=True)
    net.write_solver(name, output_dir=odir, ode_solver_source=None)
    # offsets of the rs_* scratch arrays, in reaction-then-cooling order
    fields = ["rs_%s" % r for r in sorted(net.reactions)]
    for c in sorted(net.cooling_actions):
        fields += ["cs_%s_%s" % (c, t) for t in sorted(net.cooling_actions[c].tables)]
    rs = ", ".join("offsetof(%s_data, %s)" % (name, f) for f in fields)
    harness = os.path.join(odir, "harness.cpp")
    with open(harness, "w") as f:
        f.write(HARNESS % dict(n=name, rs=rs))
    lib = os.path.join(OUT, "libref_%s.so" % tag)
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-w",
           "-I", os.path.join(HERE, "hdf5_shim"), "-I", odir,
           os.path.join(odir, "%s_solver.C" % name),
           os.path.join(REF_ROOT, "dengo", "solvers", "BE_chem_solve.C"),
           harness, "-o", lib, "-lm"]
    subprocess.check_call(cmd)
    return lib


def build_cython_driver(name="primordial"):
    """Compile the reference's rendered Cython driver (see the module
    docstring); returns the extension's directory (import
    ``<name>_solver_run`` from there, with that directory as the working
    directory so the solver finds its tables)."""
    odir = os.path.join(OUT, name)
    pyx = os.path.join(odir, "%s_solver_run.pyx" % name)
    if not os.path.exists(pyx):
        build(name)
    cpp = os.path.join(odir, "%s_solver_run.cpp" % name)
    subprocess.check_call([sys.executable, "-m", "cython", "-2", "--cplus", pyx, "-o", cpp],
                          stdout=subprocess.DEVNULL)
    so = os.path.join(odir, "%s_solver_run%s" % (name, sysconfig.get_config_var("EXT_SUFFIX")))
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
                           "-I", sysconfig.get_paths()["include"], "-I", np.get_include(),
                           "-I", os.path.join(HERE, "hdf5_shim"), "-I", odir, cpp,
                           os.path.join(odir, "%s_solver.C" % name),
                           os.path.join(REF_ROOT, "dengo", "solvers", "BE_chem_solve.C"),
                           "-o", so, "-lm"])
    return odir


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else "primordial",
                intermediate=sys.argv[2:] == ["intermediate"]))
