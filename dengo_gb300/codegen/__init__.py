"""Template rendering for the GB300 solver (the CUDA template backend).

``render_solver(net, name, output_dir, family)`` writes, for template family
``family`` (the reference's family name ``rates_and_rate_tables`` selects
this package's CUDA family), one file per suffix of that family:

    <name>_solver.cu   device functions + kernels + C entry points
    <name>_solver.h    the drop-in C header

The reference renders a fixed list of suffixes for its C++ family
(dengo/chemical_network.py:285-293); here each family declares its own.
"""

import os

import jinja2

from .spec import network_spec

TEMPLATE_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "templates")

FAMILIES = {
    "rates_and_rate_tables": ((".cu", "rates_and_rate_tables.cu.j2"),
                              (".h", "rates_and_rate_tables.h.j2"),
                              ("_main.cu", "rates_and_rate_tables_main.cu.j2"),
                              ("_run.py", "rates_and_rate_tables_run.py.j2"),
                              ("_main.py", "rates_and_rate_tables_main.py.j2")),
}
FAMILIES["cuda_be"] = FAMILIES["rates_and_rate_tables"]


def _env():
    return jinja2.Environment(loader=jinja2.FileSystemLoader(TEMPLATE_DIR),
                              keep_trailing_newline=True, undefined=jinja2.StrictUndefined)


# The engine kernels one network library holds, one translation unit each in
# the package build: (launcher, BLOCK or warps per cell, mixed precision).
ENGINE_VARIANTS = [("launch_lane", b, m) for b in (32, 64, 128) for m in ("false", "true")] + \
                  [("launch_split", w, m) for w in (2, 4) for m in ("false", "true")] + \
                  [("launch_wide", 4, m) for m in ("false", "true")]


def render_solver(net, name, output_dir, family="rates_and_rate_tables"):
    if family not in FAMILIES:
        raise KeyError("unknown solver template family %r (known: %s)"
                       % (family, ", ".join(sorted(FAMILIES))))
    spec = network_spec(net, name)
    env = _env()
    paths = []
    for suffix, tname in FAMILIES[family]:
        text = env.get_template(tname).render(s=spec, n=name, variants=ENGINE_VARIANTS)
        path = os.path.join(output_dir, "%s_solver%s" % (name, suffix))
        with open(path, "w") as f:
            f.write(text)
        paths.append(path)
    return paths
