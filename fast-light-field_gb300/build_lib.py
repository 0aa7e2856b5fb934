"""Build recipe for libflf.so (the sm_103a CUDA library behind include/flf.h).

Compiles the CUDA translation units in ``csrc/`` in parallel with nvcc for
``sm_103a`` only and links them into ``libflf.so`` next to this file (an
in-tree build; the .so is git-ignored).  ``build()`` is idempotent: it skips
work when the library is newer than every source file.
"""

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libflf.so")
OBJDIR = os.path.join(HERE, "_build")
SOURCES = ["flf_kernels.cu", "flf_api.cu", "flf_fft_part0.cu", "flf_fft_part1.cu", "flf_fft_part2.cu",
           "flf_fft_part3.cu", "flf_psf.cu", "flf_net.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


def nvcc_path():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libflf.so")


def _deps():
    files = [os.path.join(CSRC, s) for s in SOURCES]
    files += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    files.append(os.path.join(INCLUDE, "flf.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps() if os.path.exists(f))


def build(force=False, verbose=False):
    """Compile libflf.so if needed; returns its path."""
    if not force and up_to_date():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    procs = []
    objs = []
    for s in SOURCES:
        obj = os.path.join(OBJDIR, s.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc] + ARCH + FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, s), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append("$ " + " ".join(cmd) + "\n" + out.decode(errors="replace"))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
