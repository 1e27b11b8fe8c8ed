"""Builds the per-network solver libraries for sm_103a with nvcc.

Each shipped network's generated sources live in
``dengo_gb300/generated/<name>/``; ``build_network`` compiles
``<name>_solver.cu`` into ``lib<name>_solver.so`` next to it.  The FP64
engine must not contract multiply-adds (``--fmad=false``) to reproduce the
reference's arithmetic; deliberate FMAs are written as intrinsics.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
GENERATED = os.path.join(PKG, "generated")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-shared", "-Xcompiler", "-ffp-contract=off"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def network_dir(name):
    return os.path.join(GENERATED, name)


def library_path(name):
    return os.path.join(network_dir(name), "lib%s_solver.so" % name)


def build_network(name, src_dir=None, out=None, verbose=False, extra=()):
    src_dir = src_dir or network_dir(name)
    out = out or os.path.join(src_dir, "lib%s_solver.so" % name)
    src = os.path.join(src_dir, "%s_solver.cu" % name)
    cmd = [nvcc()] + ARCH_FLAGS + NVCC_FLAGS + list(extra) + [
        "-I", INCLUDE, "-I", CSRC, "-I", src_dir, src, "-o", out]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (name, res.stdout, res.stderr))
    if verbose:
        sys.stderr.write(res.stderr)
    return out


def build_all(names=None, verbose=False):
    """Every CUDA library of the package: one per shipped network plus the
    peak microbenchmark, compiled in parallel."""
    from .networks import SHIPPED_NETWORKS
    names = list(names or SHIPPED_NETWORKS)
    jobs = [lambda n=n: build_network(n, verbose=verbose) for n in names] + [build_peak]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        return [f.result() for f in [ex.submit(j) for j in jobs]]


def generate(name):
    """Re-render a shipped network's sources and tables from its definition."""
    from .networks import build_network as make_net
    net = make_net(name)
    os.makedirs(network_dir(name), exist_ok=True)
    return net.write_solver(name, output_dir=network_dir(name))


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] == "generate":
        for n in args[1:]:
            print(generate(n))
    else:
        print(build_all(args or None, verbose=True))


def build_peak():
    """The CUDA-core FMA peak microbenchmark (libdg_peak.so)."""
    out = os.path.join(PKG, "lib", "libdg_peak.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = [nvcc()] + ARCH_FLAGS + ["-O3", "-Xcompiler", "-fPIC", "-shared",
                                   os.path.join(CSRC, "dg_peak.cu"), "-o", out]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for dg_peak.cu:\n%s" % res.stderr)
    return out
