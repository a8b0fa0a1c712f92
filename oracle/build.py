"""Build recipe for the CPU oracle (test infrastructure only).

    python -m oracle.build          # both targets that can be built here

* ``oracle/_build/liboracle.so`` -- the plain-C restatement ``kernels.c``.
  Built on every machine (gcc only).
* ``oracle/_ref/libref.so`` -- the reference's own ``mermake/maxima.cu`` and
  ``mermake/blur.cu`` compiled unchanged as C++ (``ref_prelude.h`` maps the
  CUDA keywords, ``ref_driver.cpp`` runs one thread index at a time).  Built
  only where a MERMAKE checkout is present (``MERMAKE_REF`` or the default
  mount point below); nothing else reads the reference tree.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("MERMAKE_REF", "/root/reference")

LIBORACLE = os.path.join(HERE, "_build", "liboracle.so")
LIBREF = os.path.join(HERE, "_ref", "libref.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "kernels.c")
    if force or _stale(LIBORACLE, [src]):
        os.makedirs(os.path.dirname(LIBORACLE), exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp",
                               "-shared", "-fPIC", "-o", LIBORACLE, src, "-lm"])
    return LIBORACLE


def build_ref(force=False):
    """Returns the library path, or None when the reference tree is absent."""
    maxima = os.path.join(REF, "mermake", "maxima.cu")
    blur = os.path.join(REF, "mermake", "blur.cu")
    if not (os.path.exists(maxima) and os.path.exists(blur)):
        return None
    prelude = os.path.join(HERE, "ref_prelude.h")
    driver = os.path.join(HERE, "ref_driver.cpp")
    if force or _stale(LIBREF, [maxima, blur, prelude, driver]):
        os.makedirs(os.path.dirname(LIBREF), exist_ok=True)
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", LIBREF, driver,
                               "-x", "c++", "-include", prelude, maxima,
                               "-x", "c++", "-include", prelude, blur])
    return LIBREF


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
