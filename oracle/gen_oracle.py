"""ORACLE -- test infrastructure.  Renders the oracle's per-network C
(oracle/gen/<name>_oracle.c) from the network definitions, using the
reference's expression printer (sympy ccode) and statement order.

Usage: python oracle/gen_oracle.py [network ...]   (default: all shipped)
"""
import os
import sys

import jinja2

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from dengo_gb300.codegen.spec import network_spec  # noqa: E402
from dengo_gb300.networks import build_network, SHIPPED_NETWORKS  # noqa: E402


def render(name):
    net = build_network(name)
    spec = network_spec(net, name)
    env = jinja2.Environment(loader=jinja2.FileSystemLoader(HERE),
                             keep_trailing_newline=True)
    return env.get_template("network_oracle.c.j2").render(s=spec)


def main(names):
    os.makedirs(os.path.join(HERE, "gen"), exist_ok=True)
    for name in names:
        path = os.path.join(HERE, "gen", "%s_oracle.c" % name)
        with open(path, "w") as f:
            f.write(render(name))
        print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1:] or list(SHIPPED_NETWORKS))
