"""Builds the in-tree CUDA library libknightking_gb300.so for sm_103a.

Translation units compile in parallel with nvcc (one -gencode, no host-arch
flags, so the same recipe builds on x86_64 and aarch64) and link into
knightking_gb300/lib/libknightking_gb300.so.

Float arithmetic must round exactly as the reference's does: device code is
compiled with -fmad=false (no multiply-add contraction), IEEE division and
square root, no fast math; host code with -ffp-contract=off.
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libknightking_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["engine.cu", "graph.cu", "apps_first.cu", "apps_node2vec.cu", "alias_noalloc.cu", "batch.cu", "serve.cu"]
# knightking_gb300/examples/, each built into lib/libkk_example_<name>.so
EXAMPLES = ["tagwalk.cu", "dynamic_walk.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off,-O3", "-I" + INCLUDE, "-I" + CSRC,
]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _obj(src):
    return os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")


def _deps():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(PKG, "examples", f) for f in os.listdir(os.path.join(PKG, "examples"))]
    for d, _, files in os.walk(INCLUDE):
        deps += [os.path.join(d, f) for f in files]
    return deps


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _deps() + [os.path.abspath(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB

    def compile_one(src):
        path = os.path.join(CSRC, src) if not src.startswith("examples/") else os.path.join(PKG, src)
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra_flags) + ["-c", path, "-o", _obj(os.path.basename(src))]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES) + len(EXAMPLES)) as ex:
        logs = list(ex.map(compile_one, SOURCES + ["examples/" + s for s in EXAMPLES]))
    if verbose:
        for lg in logs:
            if lg:
                print(lg, file=sys.stderr)

    def link(out, objs, extra):
        tmp = out + ".tmp"
        r = subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + extra, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed for %s:\n%s%s" % (out, r.stdout, r.stderr))
        os.replace(tmp, out)

    link(LIB, [_obj(s) for s in SOURCES], [])
    # examples of the plugin API, linked against the engine library
    for s in EXAMPLES:
        name = os.path.join(LIBDIR, "libkk_example_%s.so" % os.path.splitext(s)[0])
        link(name, [_obj(s)], ["-L" + LIBDIR, "-lknightking_gb300", "-Xlinker", "-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
