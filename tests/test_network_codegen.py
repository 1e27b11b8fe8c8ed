"""Network API and code generation against the reference's expressions and
tables (tests/golden/, produced from the reference's own rendering)."""
import json
import os
import platform
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def net():
    from dengo_gb300.networks import primordial_network
    return primordial_network()


@pytest.fixture(scope="module")
def spec(net):
    from dengo_gb300.codegen.spec import network_spec
    return network_spec(net, "primordial")


@pytest.fixture(scope="module")
def ref_exprs():
    with open(os.path.join(ROOT, "tests", "golden", "primordial_expressions.json")) as f:
        return json.load(f)


def test_species_order(spec, ref_exprs):
    assert [s.name for s in spec.species] == ref_exprs["species"]
    assert [s.name for s in spec.species] == ["H2_1", "H2_2", "H_1", "H_2", "H_m0", "He_1",
                                              "He_2", "He_3", "de", "ge"]


def test_table_order(spec, ref_exprs):
    assert [t.name for t in spec.tables] == ref_exprs["tables"]
    assert len(spec.tables) == 44


def test_rhs_and_jacobian_text_equal_reference(spec, ref_exprs):
    assert spec.rhs_ref == ref_exprs["rhs"]
    assert spec.jac_ref == ref_exprs["jac"]
    assert spec.T_ref == ref_exprs["T"]
    assert spec.Tge_ref == ref_exprs["Tge"]
    assert spec.mass_density_ref == ref_exprs["density"]


def test_ge_column_is_zero(spec):
    # The reference's Jacobian has no rate-temperature terms (see
    # reaction_classes.ReactionCoefficient).
    ige = spec.ige
    assert not any(spec.jac_nonzero[ige])
    assert spec.nnz() == 54


def test_device_text_has_same_operands(spec):
    # The device printer only renames: strip "[i]", integer powers.
    import re
    for ref, dev in zip(spec.rhs_ref, spec.rhs_dev):
        r = re.sub(r"pow\(([^,()]+), (\d)\)", r"dg_ipow<\2>(\1)", ref.replace("[i]", ""))
        assert r.split("=", 1)[1] == dev.split("=", 1)[1]


def test_tables_equal_reference(net, golden):
    mine = net.rate_tables()
    names = list(golden["table_names"])
    for name, arr in mine.items():
        ref = golden["tables"][names.index(name)]
        if platform.machine() == "x86_64":
            assert np.array_equal(arr.view(np.int64), ref.view(np.int64)), name
        else:
            assert np.allclose(arr, ref, rtol=1e-13, atol=0), name


SHIPPED = ("primordial", "primordial_compton", "oxygen", "oxygen_uvb")


@pytest.mark.parametrize("name", SHIPPED)
def test_generated_sources_up_to_date(name):
    """The committed generated sources are what the templates render now."""
    from dengo_gb300.codegen import render_solver
    from dengo_gb300.networks import SHIPPED_NETWORKS, build_network
    assert SHIPPED == tuple(SHIPPED_NETWORKS)
    gen = os.path.join(ROOT, "dengo_gb300", "generated", name)
    with tempfile.TemporaryDirectory() as d:
        for p in render_solver(build_network(name), name, d):
            with open(p) as f, open(os.path.join(gen, os.path.basename(p))) as g:
                assert f.read() == g.read(), os.path.basename(p)


@pytest.mark.parametrize("name", SHIPPED)
def test_oracle_sources_up_to_date(name):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gen_oracle
    with open(os.path.join(ROOT, "oracle", "gen", "%s_oracle.c" % name)) as f:
        assert f.read() == gen_oracle.render(name)


def test_table_file_roundtrip(tmp_path):
    from dengo_gb300.tablefile import read_table_file, write_table_file
    d = {"a": np.arange(5.0), "b_c": np.array([1e-300, -0.0, np.inf])}
    write_table_file(str(tmp_path / "t.dgt"), d)
    r = read_table_file(str(tmp_path / "t.dgt"))
    assert set(r) == {"a", "b_c"}
    assert np.array_equal(r["b_c"].view(np.int64), d["b_c"].view(np.int64))


def test_write_solver_writes_all_outputs(net, tmp_path):
    init = {s: np.ones(3) for s in net.species_list()}
    paths = net.write_solver("demo", output_dir=str(tmp_path), init_values=init)
    names = sorted(os.path.basename(p) for p in paths)
    assert names == ["demo_initial_conditions.dgt", "demo_solver.cu", "demo_solver.h",
                     "demo_solver_main.cu", "demo_solver_main.py", "demo_solver_run.py",
                     "demo_tables.dgt"]
    run = open(os.path.join(str(tmp_path), "demo_solver_run.py")).read()
    assert "def run_demo(" in run and "def main_run_demo(" in run
    assert "demo_main(argc, argv)" in open(os.path.join(str(tmp_path), "demo_solver_main.cu")).read()


WRITER_CHECK = "\n".join([
    '#include "dg_tablefile.h"',
    "int main(int, char **argv) {",
    "    std::vector<std::pair<std::string, std::vector<double>>> s;",
    '    s.emplace_back("H_1", std::vector<double>{1.5, -2.25e-300, 3.0});',
    '    s.emplace_back("time", std::vector<double>(1, 4.5e13));',
    "    std::string err;",
    "    std::map<std::string, std::vector<double>> back;",
    "    if (!dg::write_table_file(argv[1], s, err)) return 1;",
    "    if (!dg::read_table_file(argv[1], back, err)) return 2;",
    '    return back["H_1"][1] == -2.25e-300 && back["time"][0] == 4.5e13 ? 0 : 3;',
    "}", ""])


def test_table_file_c_writer_round_trip(tmp_path):
    """The C++ .dgt writer (csrc/dg_tablefile.h, used by <n>_main for the
    solution file) produces what the Python reader reads."""
    import subprocess
    from dengo_gb300.tablefile import read_table_file
    src = tmp_path / "w.cpp"
    src.write_text(WRITER_CHECK)
    exe = tmp_path / "w"
    subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(ROOT, "dengo_gb300", "csrc"),
                           str(src), "-o", str(exe)])
    out = tmp_path / "sol.dgt"
    assert subprocess.call([str(exe), str(out)]) == 0
    d = read_table_file(str(out))
    assert list(d) == ["H_1", "time"] and d["H_1"][1] == -2.25e-300 and d["time"][0] == 4.5e13


def test_unknown_names_raise_the_references_exceptions():
    """Lookups of unregistered names raise dengo's exception types
    (dengo/exceptions.py), which are also KeyErrors."""
    from dengo_gb300.chemical_network import ChemicalNetwork
    from dengo_gb300.exceptions import DengoException, UnknownReaction, UnknownSpecies
    from dengo_gb300.mixin import ComparableMixin
    from dengo_gb300.reaction_classes import Species, ensure_species
    net = ChemicalNetwork()
    with pytest.raises(UnknownReaction) as e:
        net.add_reaction("no_such_reaction")
    assert isinstance(e.value, KeyError) and isinstance(e.value, DengoException)
    assert "no_such_reaction" in str(e.value)
    with pytest.raises(UnknownSpecies):
        ensure_species("no_such_species")
    assert issubclass(Species, ComparableMixin)


def test_shipped_primordial_tables_are_the_references(golden):
    """The .dgt bundle the primordial library loads holds the reference's
    tables, bit for bit."""
    from dengo_gb300.build import network_dir
    from dengo_gb300.tablefile import read_table_file
    t = read_table_file(os.path.join(network_dir("primordial"), "primordial_tables.dgt"))
    names = list(golden["table_names"])
    assert sorted(t) == sorted(names)
    for name in names:
        ref = golden["tables"][names.index(name)]
        assert np.array_equal(t[name].view(np.int64), ref.view(np.int64)), name
