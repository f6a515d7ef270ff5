"""In-tree build of libtomograpy_gb300.so (nvcc, sm_103a only).

Each CUDA translation unit under ``csrc/`` is compiled in parallel to an
object file under ``_build/`` and linked into ``libtomograpy_gb300.so`` next to
this file.  ``siddon_ref.cu`` (the reference-faithful double-precision kernel)
is compiled with ``--fmad=false`` so that no multiply-add is contracted.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtomograpy_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
UNITS = {
    "siddon_fast.cu": [],
    "siddon_ref.cu": ["--fmad=false"],
    "deterministic.cu": [],
    "reduce.cu": [],
    "noalloc.cu": [],
    "packed.cu": [],
    "packed_tuned.cu": [],
    "capi.cu": [],
}


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found: cannot build libtomograpy_gb300.so")
    return exe


def _sources():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    procs = []
    for unit, extra in UNITS.items():
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = [exe] + COMMON + extra + (["-Xptxas", "-v"] if ptxas_verbose else []) + \
            ["-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((unit, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                                  text=True)))
    objs = []
    errors = []
    for unit, obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append("%s:\n%s" % (unit, out[-6000:]))
        elif (verbose or ptxas_verbose) and out:
            print(out, file=sys.stderr)
        objs.append(obj)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_verbose="-v" in sys.argv))
