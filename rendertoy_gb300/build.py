"""Build librtx.so in-tree: CUDA kernels for sm_103a plus the host C ABI.

    python -m rendertoy_gb300.build          # or rendertoy_gb300.build.build()

Kernels are compiled with --fmad=false: no multiply-add is contracted unless
the source asks for it (__fmaf_rn), so the arithmetic of the hot path rounds
as RenderToy's does.  Host files use -ffp-contract=off for the same reason.
The CUDA runtime is linked statically, so the library does not depend on the
libcudart that another framework in the process may have loaded.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librtx.so")
COMPAT_LIB = os.path.join(HERE, "librendertoy_compat.so")
COMPAT_INC = os.path.join(HERE, "compat", "include")
COMPAT_SRC = os.path.join(HERE, "compat", "src")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc():
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    return p


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _deps_mtime():
    return max(os.path.getmtime(os.path.join(d, f))
               for d in (CSRC, os.path.join(ROOT, "include"))
               for f in os.listdir(d) if f.endswith((".cu", ".cuh", ".h", ".cpp")))


def _compile(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_compat(force: bool = False) -> str:
    """The RenderToy-compatible C++ API (compat/) as librendertoy_compat.so,
    linked against librtx.so."""
    build(force=force)
    srcs = [os.path.join(COMPAT_SRC, f) for f in sorted(os.listdir(COMPAT_SRC)) if f.endswith(".cpp")]
    deps = srcs + [os.path.join(COMPAT_INC, "RenderToy", f) for f in os.listdir(os.path.join(COMPAT_INC, "RenderToy"))]
    if not force and os.path.exists(COMPAT_LIB) and \
            os.path.getmtime(COMPAT_LIB) >= max(max(os.path.getmtime(d) for d in deps), os.path.getmtime(LIB)):
        return COMPAT_LIB
    tmp = COMPAT_LIB + ".tmp"
    _compile(["g++", "-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-o", tmp,
              "-I" + COMPAT_INC, *srcs, "-L" + HERE, "-lrtx", "-Wl,-rpath,$ORIGIN",
              "-Wl,--no-undefined"])
    os.replace(tmp, COMPAT_LIB)
    return COMPAT_LIB


def compile_app(src: str, out: str) -> str:
    """Compile a RenderToy application against the compatible API."""
    build_compat()
    _compile(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-I" + COMPAT_INC, src, "-o", out,
              "-L" + HERE, "-lrendertoy_compat", "-lrtx", "-Wl,-rpath," + HERE])
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link librtx.so; returns its path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    cu, cpp = _sources()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    cmds = []
    objs = []
    for f in cu:
        o = os.path.join(OBJ, f + ".o")
        objs.append(o)
        extra = os.environ.get("RTX_NVCC_FLAGS", "").split()
        cmds.append([_nvcc(), *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", *extra,
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
                     *inc, "-c", os.path.join(CSRC, f), "-o", o])
    # macro definitions among the extra flags reach the host sources too, so
    # that host and device code never disagree on a layout constant
    host_defs = [f for f in os.environ.get("RTX_NVCC_FLAGS", "").split() if f.startswith(("-D", "-U"))]
    for f in cpp:
        o = os.path.join(OBJ, f + ".o")
        objs.append(o)
        cmds.append(["g++", "-O2", "-fPIC", "-ffp-contract=off", "-std=c++17", "-fopenmp", *host_defs,
                     "-I" + os.path.join(CUDA_HOME, "include"), *inc, "-c",
                     os.path.join(CSRC, f), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        outs = list(ex.map(_compile, cmds))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _compile(["g++", "-shared", "-o", tmp, *objs, "-L" + os.path.join(CUDA_HOME, "lib64"),
              "-Wl,--no-undefined", "-lcudart_static", "-ldl", "-lrt", "-lpthread", "-fopenmp"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_compat())
