"""Build libbubbledyn.so (the C ABI of include/bubbledyn.h) for sm_103a, and
the command-line drivers that call it.

Each csrc/*.cu is compiled by nvcc in parallel into bubbledynamics_gb300/_build/
and linked into bubbledynamics_gb300/lib/libbubbledyn.so; each cli/*.cpp is
compiled by the host C++ compiler into bubbledynamics_gb300/bin/ and linked
against that library (all git-ignored).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libbubbledyn.so")
INCLUDE = os.path.join(HERE, "..", "include")
CLI_SRC = os.path.join(HERE, "cli")
BINDIR = os.path.join(HERE, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "-diag-suppress", "550", "-I", INCLUDE]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    if _stale(obj, [src] + _headers()) or extra:
        cmd = [nvcc()] + ARCH + NVFLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False, extra=None):
    """Compile and link; returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = list(extra or [])
    if force:
        for o in glob.glob(os.path.join(OBJ, "*.o")):
            os.remove(o)
    srcs = _sources()
    jobs = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if _stale(LIB, objs) or force:
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    build_cli()
    return LIB


def cli_path(name):
    return os.path.join(BINDIR, name)


def build_cli():
    """The command-line drivers (bd_westervelt, bd_spiral, bd_gilmore): host
    C++ against the C ABI only, run-path set to the library's directory."""
    os.makedirs(BINDIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    hdrs = [os.path.join(CLI_SRC, "cli_common.h"), os.path.join(INCLUDE, "bubbledyn.h")]

    def one(src):
        exe = cli_path(os.path.basename(src)[:-4])
        if _stale(exe, [src, LIB] + hdrs):
            cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, src, "-o", exe, "-L", LIBDIR, "-lbubbledyn",
                   "-Wl,-rpath,$ORIGIN/../lib"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("C++ driver build failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return exe

    srcs = sorted(glob.glob(os.path.join(CLI_SRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max(1, len(srcs))) as ex:
        return list(ex.map(one, srcs))


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
