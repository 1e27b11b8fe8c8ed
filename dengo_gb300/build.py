"""Builds the per-network solver libraries for sm_103a with nvcc.

Each shipped network's generated sources live in
``dengo_gb300/generated/<name>/``; ``build_network`` compiles
``<name>_solver.cu`` -- once for the entry points and once per engine variant,
in parallel -- into ``lib<name>_solver.so`` next to it.  The FP64
engine must not contract multiply-adds (``--fmad=false``) to reproduce the
reference's arithmetic; deliberate FMAs are written as intrinsics.
"""

import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
GENERATED = os.path.join(PKG, "generated")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def network_dir(name):
    return os.path.join(GENERATED, name)


def library_path(name):
    return os.path.join(network_dir(name), "lib%s_solver.so" % name)


def _run(cmd, what, verbose):
    if verbose:
        print(" ".join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (what, res.stdout, res.stderr))
    if verbose:
        sys.stderr.write(res.stderr)


class _NetworkBuild:
    """The translation units of one network library: the entry points
    (-DDG_SPLIT_KERNELS) and one unit per engine variant
    (-DDG_KERNEL_PART=k), linked into lib<name>_solver.so."""

    def __init__(self, name, src_dir, out, tmp, verbose, extra):
        from .codegen import ENGINE_VARIANTS
        self.name, self.out, self.verbose = name, out, verbose
        src = os.path.join(src_dir, "%s_solver.cu" % name)
        base = [nvcc()] + (["-Xptxas=-v"] if verbose else []) + ARCH_FLAGS + NVCC_FLAGS + \
            list(extra) + ["-I", INCLUDE, "-I", CSRC, "-I", src_dir, "-c", src]
        defs = ["-DDG_SPLIT_KERNELS"] + ["-DDG_KERNEL_PART=%d" % k
                                         for k in range(len(ENGINE_VARIANTS))]
        self.objs = [os.path.join(tmp, "%s_%d.o" % (name, i)) for i in range(len(defs))]
        self.compiles = [base + [d, "-o", o] for d, o in zip(defs, self.objs)]

    def compile(self, i):
        _run(self.compiles[i], "%s (unit %d)" % (self.name, i), self.verbose)

    def link(self):
        _run([nvcc()] + ARCH_FLAGS + ["-shared", "-Xcompiler", "-fPIC"] + self.objs +
             ["-o", self.out], "%s (link)" % self.name, self.verbose)
        return self.out


def _build(builds, extra_jobs=(), verbose=False):
    with tempfile.TemporaryDirectory(prefix="dg_build_") as tmp:
        nb = [b(tmp) for b in builds]
        units = [(b, i) for b in nb for i in range(len(b.compiles))]
        workers = max(2, min(len(units) + len(extra_jobs), os.cpu_count() or 4))
        with ThreadPoolExecutor(max_workers=workers) as ex:
            extra = [ex.submit(j) for j in extra_jobs]
            for f in [ex.submit(b.compile, i) for b, i in units]:
                f.result()
            outs = [f.result() for f in [ex.submit(b.link) for b in nb]]
            return outs + [f.result() for f in extra]


def build_network(name, src_dir=None, out=None, verbose=False, extra=()):
    """lib<name>_solver.so from generated/<name>/<name>_solver.cu (its units
    compiled in parallel)."""
    src_dir = src_dir or network_dir(name)
    out = out or os.path.join(src_dir, "lib%s_solver.so" % name)
    return _build([lambda tmp: _NetworkBuild(name, src_dir, out, tmp, verbose, extra)],
                  verbose=verbose)[0]


def build_all(names=None, verbose=False):
    """Every CUDA library of the package: one per shipped network plus the
    peak microbenchmark, all translation units compiled in parallel."""
    from .networks import SHIPPED_NETWORKS
    names = list(names or SHIPPED_NETWORKS)
    builds = [lambda tmp, n=n: _NetworkBuild(n, network_dir(n), library_path(n), tmp, verbose, ())
              for n in names]
    return _build(builds, extra_jobs=[build_peak], verbose=verbose)


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
