"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``libhodlr_oracle.so`` -- the C restatement in ``hodlr_oracle.c``; built on
  any machine with gcc (x86_64 or aarch64).
* ``libhsolve_blas.so`` -- ``hsolve_blas.c``: hsolve restated with the BLAS
  calls it makes, bound at run time to scipy's bundled OpenBLAS, and its
  threaded form (the CPU baseline); built on any machine with gcc.
* ``_ref/libhsolve_ref.so`` -- fastSolver2's own ``hsolve``
  (src/tasks/leaf_solve.cc:73-154) compiled verbatim.  The lines are streamed
  out of the read-only reference checkout with ``sed`` straight into g++
  (no copy is written), prefixed with ``ref_shim.h`` and linked to scipy's
  bundled OpenBLAS for ``dgemm_``/``dgesv_``.  Only possible where the
  reference checkout and scipy's OpenBLAS are both present; otherwise skipped.

Run ``python oracle/build.py`` or call :func:`build`.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where the fastSolver2 checkout lives (read only); FASTSOLVER2_REFERENCE overrides
REF_ROOT = os.environ.get("FASTSOLVER2_REFERENCE", "/root/reference")
REF_FILE = os.path.join(REF_ROOT, "src", "tasks", "leaf_solve.cc")
HSOLVE_LINES = (73, 154)

ORACLE_SO = os.path.join(HERE, "libhodlr_oracle.so")
BLAS_SO = os.path.join(HERE, "libhsolve_blas.so")
REF_SO = os.path.join(HERE, "_ref", "libhsolve_ref.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "hodlr_oracle.c")
    if force or _stale(ORACLE_SO, [src, __file__]):
        cmd = ["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               "-fvisibility=hidden", src, "-o", ORACLE_SO + ".tmp", "-lm"]
        subprocess.check_call(cmd)
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_blas_port(force=False):
    src = os.path.join(HERE, "hsolve_blas.c")
    if force or _stale(BLAS_SO, [src, __file__]):
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               "-fvisibility=hidden", src, "-o", BLAS_SO + ".tmp", "-ldl", "-lm"]
        subprocess.check_call(cmd)
        os.replace(BLAS_SO + ".tmp", BLAS_SO)
    return BLAS_SO


def scipy_openblas():
    """Path of scipy's bundled OpenBLAS, or None."""
    return _scipy_openblas()


def _scipy_openblas():
    try:
        import scipy
    except ImportError:
        return None
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    hits = sorted(glob.glob(os.path.join(libdir, "libscipy_openblas*.so")))
    return hits[0] if hits else None


def build_reference(force=False):
    """Compile the verbatim reference hsolve.  Returns the .so path or None."""
    if not os.path.exists(REF_FILE):
        return None
    blas = _scipy_openblas()
    if blas is None:
        return None
    lo, hi = HSOLVE_LINES
    body = subprocess.check_output(["sed", "-n", f"{lo},{hi}p", REF_FILE]).decode()
    first = body.lstrip().splitlines()[0]
    if not (first.startswith("void hsolve") and body.rstrip().endswith("}")):
        raise RuntimeError("hsolve is no longer at %s:%d-%d" % (REF_FILE, lo, hi))
    shim = os.path.join(HERE, "ref_shim.h")
    stubs = os.path.join(HERE, "ref_blas.cc")
    if not force and not _stale(REF_SO, [REF_FILE, shim, stubs, __file__]):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    obj = REF_SO + ".hsolve.o"
    cc = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-w"]
    subprocess.run(cc + ["-include", shim, "-x", "c++", "-", "-c", "-o", obj],
                   input=body.encode(), check=True)
    libdir = os.path.dirname(blas)
    subprocess.check_call(cc + ["-shared", stubs, obj, "-o", REF_SO + ".tmp",
                                blas, "-Wl,-rpath," + libdir])
    os.replace(REF_SO + ".tmp", REF_SO)
    os.remove(obj)
    return REF_SO


def build(force=False):
    build_oracle(force)
    build_blas_port(force)
    try:
        build_reference(force)
    except (subprocess.CalledProcessError, OSError) as e:  # reference is optional
        print("oracle: reference hsolve not built:", e, file=sys.stderr)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(ORACLE_SO, REF_SO if os.path.exists(REF_SO) else "(no reference build)")
