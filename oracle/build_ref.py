"""Build recipe for the *reference's own* Siddon C kernel (test infrastructure).

This script compiles TomograPy's ``tomograpy/C_siddon.c.template`` -- exactly as
the reference ships it -- into CPython extension modules under ``oracle/_ref/``.
It is used only to pin the oracle (``oracle/siddon_oracle.c``) and to generate
the golden fixtures under ``tests/golden/``.  Nothing in the product imports it.

Steps (mirroring what ``tomograpy/parse_templates.py:11-34`` and
``setup.py:17-22`` do, without running the reference's build system):

1. read the template from the reference checkout (read-only),
2. ``%``-substitute ``ctype``/``obstacle``/``pj``/``suffix`` for each of the
   variants requested (the same substitution keys as
   ``tomograpy/parse_templates.py:19-26,62-63``) into a temporary directory,
3. compile each expansion with a small Python-3 module-init shim (the template's
   ``init_C_siddon...``/``Py_InitModule`` entry point is Python-2 only,
   ``tomograpy/C_siddon.c.template:70,174-178``); the shim includes the
   expanded source unchanged and adds a ``PyInit_`` function around its method
   table,
4. write only the resulting ``.so`` files into ``oracle/_ref/``.

The expanded sources stay in the temporary directory; ``oracle/_ref/`` is
git-ignored.  Run: ``python oracle/build_ref.py [--reference PATH]`` (default:
``$TOMOGRAPY_REFERENCE``, else a checkout named ``reference`` beside the
repository).
"""
import argparse
import os
import subprocess
import sys
import sysconfig
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference checkout: $TOMOGRAPY_REFERENCE, else a directory named
# "reference" beside this repository's root.
DEFAULT_REFERENCE = os.environ.get("TOMOGRAPY_REFERENCE") or \
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

CTYPES = ("float", "double")
OBSTACLES = ("none", "sun")
PJS = ("pj", "bpj", "pjt", "bpjt")

SHIM = r"""
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <numpy/arrayobject.h>
/* The expanded template includes "arrayobject.h" again (guarded) and defines a
   Python-2 init function; neutralise the two Python-2-only calls inside it. */
#undef import_array
#define import_array()
#define Py_InitModule(name, methods) ((PyObject *)0)
#include "%(src)s"
static struct PyModuleDef tg_ref_moddef = {
  PyModuleDef_HEAD_INIT, "_C_siddon%(suffix)s", NULL, -1, _C_siddon%(suffix)sMethods
};
PyMODINIT_FUNC PyInit__C_siddon%(suffix)s(void)
{
  PyObject *m;
  if (_import_array() < 0) return NULL;
  m = PyModule_Create(&tg_ref_moddef);
  return m;
}
"""


def variants(ctypes=CTYPES, obstacles=OBSTACLES, pjs=PJS):
    for c in ctypes:
        for o in obstacles:
            for p in pjs:
                yield {"ctype": c, "obstacle": o, "pj": p,
                       "suffix": "_%s_%s_%s" % (c, o, p)}


def _compile(args):
    tmp, template, v, numpy_inc, py_inc = args
    values = dict(v)
    values.update({"f": "%f", "d": "%d"})
    src = os.path.join(tmp, "C_siddon%s.c" % v["suffix"])
    with open(src, "w") as f:
        f.write(template % values)
    shim = os.path.join(tmp, "shim%s.c" % v["suffix"])
    with open(shim, "w") as f:
        f.write(SHIM % {"src": src, "suffix": v["suffix"]})
    out = os.path.join(OUT, "_C_siddon%s%s" % (v["suffix"], sysconfig.get_config_var("EXT_SUFFIX")))
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-fgnu89-inline",
           "-w", "-I", py_inc, "-I", numpy_inc, "-I", os.path.join(numpy_inc, "numpy"),
           shim, "-o", out, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed for %s:\n%s" % (v["suffix"], r.stderr[-4000:]))
    return out


def reference_present(reference=DEFAULT_REFERENCE):
    """True where the reference checkout is available (not on the GPU host)."""
    return os.path.isdir(os.path.join(reference, "tomograpy"))


def build(reference=DEFAULT_REFERENCE, quiet=False):
    """Compile all 16 reference variants into oracle/_ref/. Returns the list of .so paths."""
    import numpy
    tpath = os.path.join(reference, "tomograpy", "C_siddon.c.template")
    if not os.path.isfile(tpath):
        raise FileNotFoundError(tpath)
    with open(tpath) as f:
        template = f.read()
    os.makedirs(OUT, exist_ok=True)
    numpy_inc = numpy.get_include()
    py_inc = sysconfig.get_paths()["include"]
    with tempfile.TemporaryDirectory() as tmp:
        jobs = [(tmp, template, v, numpy_inc, py_inc) for v in variants()]
        with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_compile, jobs))
    if not quiet:
        print("built %d reference modules into %s" % (len(outs), OUT))
    return outs


def load(ctype="double", obstacle="sun", pj="pj"):
    """Import one compiled reference module from oracle/_ref/ (build() first)."""
    import importlib
    if OUT not in sys.path:
        sys.path.insert(0, OUT)
    return importlib.import_module("_C_siddon_%s_%s_%s" % (ctype, obstacle, pj))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    a = ap.parse_args()
    build(a.reference)
