"""The code generator's parsers for the wide engine's lane-parallel forms
(dengo_gb300/codegen/spec.py): sums of signed products (sop_parse /
sop_tables), the temperature's term lists (temperature_lanes) and the
shared-subexpression part balancing (balance_shared).  Pure Python."""
import pytest

from dengo_gb300.codegen.spec import (balance_shared, sop_parse, temperature_lanes)

NAMES = {"k01", "k02", "H_1", "H_2", "de"}


def test_sop_parse_accepts_flat_sums_of_products():
    t = sop_parse("-k01*H_1*de + 2*k02*dg_ipow<2>(H_2) - k02*H_1", NAMES)
    assert t == [(-1, [("name", "k01"), ("name", "H_1"), ("name", "de")]),
                 (1, [("lit", "2"), ("name", "k02"), ("pow", 2, "H_2")]),
                 (-1, [("name", "k02"), ("name", "H_1")])]
    assert sop_parse("k01", NAMES) == [(1, [("name", "k01")])]


@pytest.mark.parametrize("expr", ["k01*(H_1 + H_2)", "k01*H_1/de", "k01*exp(H_1)",
                                  "k01*X_9", "k01*H_1 +", "dg_ipow<9>(H_1)", "k01**H_1",
                                  "-(k01*H_1)"])
def test_sop_parse_rejects_other_forms(expr):
    assert sop_parse(expr, NAMES) is None


def test_shipped_networks_have_tables_and_temperature_lanes():
    from dengo_gb300.codegen.spec import network_spec
    from dengo_gb300.networks import build_network
    for name in ("primordial", "oxygen"):
        s = network_spec(build_network(name), name)
        assert s.t_lanes is not None
        assert s.sop is not None and s.sop["rhs_entries"] and s.sop["jac_entries"]
        # every structurally nonzero entry is tabled or left to the scalar parts
        nnz = sum(1 for v in range(s.N) for q in range(s.N) if s.jac_nonzero[v][q])
        assert len(s.sop["jac_entries"]) + len(s.sop["jac_rest"]) == nnz
        assert len(s.sop["rhs_entries"]) + len(s.sop["rhs_rest"]) == s.N


def test_temperature_lanes_rejects_another_form():
    from collections import namedtuple
    Sp = namedtuple("Sp", "name index")
    sp = [Sp("H_1", 0), Sp("de", 1), Sp("ge", 2)]
    ok = temperature_lanes(sp, "1.0079400000000001*H_1",
                           "density*ge*mh/(kb*(dg_div(H_1, gm1, rgm1) + dg_div(de, gm1, rgm1)))",
                           "density*mh/(kb*(dg_div(H_1, gm1, rgm1) + dg_div(de, gm1, rgm1)))")
    assert ok == {"density": [(0, "1.0079400000000001")], "quot": [0, 1]}
    assert temperature_lanes(sp, "H_1*H_1", "density*ge*mh/(kb*(dg_div(H_1, gm1, rgm1)))",
                             "density*mh/(kb*(dg_div(H_1, gm1, rgm1)))") is None
    assert temperature_lanes(sp, "H_1", "density*ge*mh/(kb*(H_1/gm1))",
                             "density*mh/(kb*(H_1/gm1))") is None


def test_balance_shared_no_worse_than_plain_balance_on_the_network():
    """Each part's cost counted with shared subexpressions once (as the
    compiler computes them): the shared-aware partition of the primordial
    Jacobian is no costlier, in its largest part and in total, than the
    plain longest-first partition by per-entry cost."""
    import re
    from dengo_gb300.codegen.spec import _cx_nodes, _cx_parse, balance, network_spec
    from dengo_gb300.networks import build_network
    s = network_spec(build_network("primordial"), "primordial")
    texts = [s.jac_dev[v][q] for v in range(s.N) for q in range(s.N)]

    def nodes(t):
        acc = {}
        _cx_nodes(_cx_parse(re.match(r"^\s*jv = (.*?);", t, re.S).group(1)), acc)
        return acc

    def loads(part, n):
        out = []
        for p in range(n):
            acc = {}
            for t, pt in zip(texts, part):
                if t is not None and pt == p:
                    acc.update(nodes(t))
            out.append(sum(acc.values()))
        return out

    own = [0.5 if t is None else sum(nodes(t).values()) + 4.0 for t in texts]
    for n in (2, 4):
        shared, plain = loads(balance_shared(texts, n), n), loads(balance(own, n), n)
        assert max(shared) <= max(plain) and sum(shared) <= sum(plain)
