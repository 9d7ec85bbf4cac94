"""Make the reference (PythonOT/POT) importable in a build container.

Only the golden-fixture generator (``gen_golden.py``) uses this; nothing that
runs on the GPU machine does, because the reference tree is not present there.

Recipe:
  1. copy the read-only reference tree into ``baseline/_ref/pot`` (git-ignored);
  2. build the two Cython extensions the package imports at start-up
     (``ot.lp.emd_wrap`` and ``ot.partial.partial_cython``) in place;
  3. insert a stub for ``ot.bsp.bsp_wrap``, whose Eigen submodule is not
     vendored in the reference tree, before ``import ot``.
"""
import os
import shutil
import subprocess
import sys
import types

REF_SRC = os.environ.get("POT_REFERENCE_SRC")  # the read-only reference tree: required, no default
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DEST = os.path.join(REPO, "baseline", "_ref", "pot")

_SETUP = r'''
import numpy
from setuptools import setup, Extension
from Cython.Build import cythonize
setup(name="pot_ref_min", ext_modules=cythonize([
    Extension("ot.lp.emd_wrap", ["ot/lp/emd_wrap.pyx", "ot/lp/EMD_wrapper.cpp"],
              language="c++", include_dirs=[numpy.get_include(), "ot/lp"],
              extra_compile_args=["-O3", "-fopenmp"], extra_link_args=["-fopenmp"]),
    Extension("ot.partial.partial_cython", ["ot/partial/partial_cython.pyx"],
              language="c++", include_dirs=[numpy.get_include(), "ot/partial"]),
], language_level=3))
'''


def build():
    if os.path.exists(os.path.join(DEST, "ot", "__init__.py")):
        have = [f for f in os.listdir(os.path.join(DEST, "ot", "lp")) if f.startswith("emd_wrap") and f.endswith(".so")]
        if have:
            return DEST
    if not REF_SRC or not os.path.isdir(REF_SRC):
        raise RuntimeError("set POT_REFERENCE_SRC to the reference (PythonOT/POT) source tree; got %r" % REF_SRC)
    if os.path.exists(DEST):
        shutil.rmtree(DEST)
    shutil.copytree(REF_SRC, DEST, ignore=shutil.ignore_patterns(".git", "docs", "data", "examples"))
    subprocess.check_call(["chmod", "-R", "u+w", DEST])
    with open(os.path.join(DEST, "_setup_min.py"), "w") as f:
        f.write(_SETUP)
    subprocess.check_call([sys.executable, "_setup_min.py", "build_ext", "--inplace"], cwd=DEST,
                          stdout=subprocess.DEVNULL)
    return DEST


def import_ot():
    dest = build()
    if "ot.bsp.bsp_wrap" not in sys.modules:
        stub = types.ModuleType("ot.bsp.bsp_wrap")

        def _na(*a, **k):
            raise NotImplementedError("BSP-OT needs Eigen, which is not vendored")

        stub.bsp_solve_c = _na
        stub.merge_bijections_c = _na
        sys.modules["ot.bsp.bsp_wrap"] = stub
    if dest not in sys.path:
        sys.path.insert(0, dest)
    import ot  # noqa: E402
    return ot


if __name__ == "__main__":
    ot = import_ot()
    print(ot.__version__, ot.__file__)
