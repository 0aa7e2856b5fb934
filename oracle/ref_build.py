"""Build recipe for the reference's own C++/FFTW CPU path (test infrastructure).

The reference's production CPU projector is the CPython extension
``py_light_field`` (py_light_field/py_light_field.cpp with its ``common/``
helpers) linked against the FFTW 3.3.8 sources it vendors
(py_light_field/fftw-3.3.8.tar.gz), driven from Python by
``projector.Projector_allC`` and ``lfdeconv.DeconvRL`` (projector.py:798-896,
lfdeconv.py:72-202).  This file builds that path from the reference's sources
and loads it; it is the CPU baseline that bench.py times beside the GPU path.
Nothing in the GB300 library imports it.

Layout, all under ``oracle/_ref/`` (git-ignored, so no reference source enters
the repository's history; it still travels with the working tree to a GPU
machine, which has no copy of the reference):

* ``src/``   copies of the reference files the path needs, staged from the
  reference checkout given to ``stage`` (the C++ sources, the FFTW tarball and
  the Python modules ``projector``, ``lfdeconv``, ``psfmatrix``,
  ``special_fftconvolve``, ``myfft``, ``jutils``, ``lfimage``);
* ``build-<machine>/``  FFTW configured as the reference's setup.py does
  (``--enable-float --enable-threads``, py_light_field/setup.py:11-17) and
  the extension compiled by one g++ command with the reference's flags
  (``-O3 -std=c++11 -flax-vector-conversions``, setup.py:42-47).  The
  reference passes ``CFLAGS=-fPIC``, which makes FFTW's configure drop its own
  optimisation flags; this recipe passes ``-fPIC -O2`` so that the baseline is
  not slowed by an unoptimised FFTW.  One build per machine type, since the
  GPU machines are aarch64.

Usage (in a checkout of the reference): ``python oracle/ref_build.py
/path/to/reference`` stages and builds; ``load()`` returns the reference's
modules with stand-ins for the packages its import lines name but this path
never calls (h5py, tifffile, generate_psf, and psutil / tqdm where missing).
"""

import os
import platform
import shutil
import subprocess
import sys
import sysconfig
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
SRC = os.path.join(REF, "src")
PY_MODULES = ["projector.py", "lfdeconv.py", "psfmatrix.py", "special_fftconvolve.py", "myfft.py", "jutils.py",
              "lfimage.py"]
CPP_SOURCES = ["py_light_field.cpp", "common/jPythonArray.cpp", "common/jPythonCommon.cpp", "common/jMutex.cpp",
               "common/jAssert.cpp", "common/DebugPrintf_Unix.cpp"]
FFTW = "fftw-3.3.8"


def build_dir():
    return os.path.join(REF, "build-" + platform.machine())


def ext_path():
    return os.path.join(build_dir(), "py_light_field" + sysconfig.get_config_var("EXT_SUFFIX"))


def staged():
    return os.path.exists(os.path.join(SRC, "python", "projector.py")) and \
        os.path.exists(os.path.join(SRC, "py_light_field", FFTW + ".tar.gz"))


def stage(ref_dir):
    """Copy the reference files the CPU path needs into oracle/_ref/src."""
    if not os.path.isdir(ref_dir):
        raise FileNotFoundError("no reference checkout at %s" % ref_dir)
    dst_py = os.path.join(SRC, "python")
    dst_c = os.path.join(SRC, "py_light_field")
    os.makedirs(dst_py, exist_ok=True)
    os.makedirs(os.path.join(dst_c, "common"), exist_ok=True)
    for m in PY_MODULES:
        shutil.copy2(os.path.join(ref_dir, m), os.path.join(dst_py, m))
    src_c = os.path.join(ref_dir, "py_light_field")
    shutil.copy2(os.path.join(src_c, FFTW + ".tar.gz"), os.path.join(dst_c, FFTW + ".tar.gz"))
    shutil.copy2(os.path.join(src_c, "py_light_field.cpp"), os.path.join(dst_c, "py_light_field.cpp"))
    for f in os.listdir(os.path.join(src_c, "common")):
        if f.endswith((".cpp", ".h")):
            shutil.copy2(os.path.join(src_c, "common", f), os.path.join(dst_c, "common", f))


def _run(cmd, cwd, log):
    with open(log, "ab") as f:
        r = subprocess.run(cmd, cwd=cwd, stdout=f, stderr=subprocess.STDOUT, shell=isinstance(cmd, str))
    if r.returncode != 0:
        raise RuntimeError("reference build step failed (%s); see %s" % (cmd, log))


def build(verbose=False):
    """Build FFTW and the extension for this machine if not built yet; returns the .so path."""
    so = ext_path()
    if os.path.exists(so):
        return so
    if not staged():
        raise FileNotFoundError("reference sources are not staged in %s (run oracle/ref_build.py with the "
                                "reference folder first)" % SRC)
    bd = build_dir()
    os.makedirs(bd, exist_ok=True)
    log = os.path.join(bd, "build.log")
    jobs = str(os.cpu_count() or 4)
    fftw = os.path.join(bd, FFTW)
    lib = os.path.join(fftw, ".libs", "libfftw3f.a")
    if not os.path.exists(lib):
        if os.path.exists(fftw):
            shutil.rmtree(fftw)
        _run(["tar", "-xzf", os.path.join(SRC, "py_light_field", FFTW + ".tar.gz")], bd, log)
        _run(["./configure", "CFLAGS=-fPIC -O2", "--enable-float", "--enable-threads", "--disable-fortran"], fftw, log)
        _run(["make", "-j" + jobs], fftw, log)
    import numpy
    csrc = os.path.join(SRC, "py_light_field")
    # the extension includes "fftw-3.3.8/api/fftw3.h" relative to its own folder
    link = os.path.join(csrc, FFTW)
    if not os.path.exists(os.path.join(link, "api", "fftw3.h")):
        os.makedirs(os.path.join(link, "api"), exist_ok=True)
        shutil.copy2(os.path.join(fftw, "api", "fftw3.h"), os.path.join(link, "api", "fftw3.h"))
    cmd = ["g++", "-O3", "-std=c++11", "-flax-vector-conversions", "-fPIC", "-shared",
           "-I" + sysconfig.get_paths()["include"], "-I" + numpy.get_include()]
    cmd += [os.path.join(csrc, s) for s in CPP_SOURCES]
    cmd += [os.path.join(fftw, "threads", ".libs", "libfftw3f_threads.a"), lib, "-lpthread", "-o", so + ".tmp"]
    _run(cmd, csrc, log)
    os.replace(so + ".tmp", so)
    if verbose:
        print("built", so, flush=True)
    return so


def _stub(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


def load():
    """(projector, lfdeconv, psfmatrix, py_light_field) of the reference, built for this machine."""
    so = build()
    for name in ("h5py", "tifffile", "generate_psf", "light_field_integrands"):
        sys.modules.setdefault(name, _stub(name))
    try:
        import psutil  # noqa: F401
    except ImportError:
        sys.modules["psutil"] = _stub("psutil", cpu_count=lambda logical=True: os.cpu_count(),
                                      virtual_memory=lambda: (0, 0, 0, 0))
    try:
        import tqdm.auto  # noqa: F401
    except ImportError:
        def tq(it=None, *a, **k):
            return it
        auto = _stub("tqdm.auto", tqdm=tq)
        sys.modules["tqdm"] = _stub("tqdm", tqdm=tq, auto=auto)
        sys.modules["tqdm.auto"] = auto
    import importlib.util
    spec = importlib.util.spec_from_file_location("py_light_field", so)
    plf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(plf)
    sys.modules["py_light_field"] = plf
    py = os.path.join(SRC, "python")
    if py not in sys.path:
        sys.path.insert(0, py)
    import projector
    import lfdeconv
    import psfmatrix
    return projector, lfdeconv, psfmatrix, plf


if __name__ == "__main__":
    if len(sys.argv) == 2:
        stage(sys.argv[1])
    elif not staged():
        sys.exit(__doc__)
    print(build(verbose=True))
