import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "primordial_golden.npz")))


@pytest.fixture(scope="session")
def tables_in_order(golden):
    """The golden tables in the solver's table order."""
    import json
    with open(os.path.join(ROOT, "tests", "golden", "primordial_expressions.json")) as f:
        order = json.load(f)["tables"]
    names = list(golden["table_names"])
    return [golden["tables"][names.index(n)] for n in order]


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle("primordial")


@pytest.fixture(scope="session")
def solver():
    """The GPU solver library (built on demand); GPU tests only."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from dengo_gb300.build import build_network, library_path
    if not os.path.exists(library_path("primordial")):
        build_network("primordial")
    from dengo_gb300.runtime import Solver
    return Solver("primordial")


def write_report(name, data):
    """Write ``data`` as JSON to ``$DENGO_REPORT_DIR/<name>.json`` when that
    variable is set (measurement runs); tests do nothing otherwise."""
    import json
    out = os.environ.get("DENGO_REPORT_DIR")
    if not out:
        return
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(out, name + ".json"), "w") as f:
        json.dump(data, f, indent=1)


def species_error_report(names, err, conv_cells, tol):
    """Per species: max and median floored relative error over the converged
    cells and the fraction of them within ``tol``."""
    import numpy as np
    rep = {"cells": int(conv_cells), "tol": tol, "species": {}}
    for k, nm in enumerate(names):
        e = err[:, k]
        rep["species"][nm] = {"max": float(e.max(initial=0.0)),
                              "median": float(np.median(e)) if len(e) else 0.0,
                              "frac_within_tol": float(np.mean(e <= tol)) if len(e) else 1.0}
    return rep
