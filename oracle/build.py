"""Build recipe of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

  oracle/_build/libbdoracle.so  the FP64 restatement (bd_oracle.cpp)
  oracle/_ref/libbdref.so       the reference's own kernel code compiled for the
                                host (ref_harness.cpp), built from the kernel
                                sections of the reference files, which are
                                extracted by line range into oracle/_ref/src/.

Both outputs are git-ignored.  The extraction needs the reference tree (the
BD_REFERENCE_DIR environment variable, else a directory named "reference"
beside this repository); where it is absent but
oracle/_ref/src/ already holds the extracted sections (a copy of this working
tree on another machine), the library is compiled from those.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: BD_REFERENCE_DIR, else a "reference" directory beside this repository
REF_DIR = os.environ.get("BD_REFERENCE_DIR", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
REF_FILES = {
    "W": "Westervelt_relax_fft_Pressure_Energy.cu",
    "T": "Westervelt_Temperature_SquareSpiral.cu",
    "G": "Gilmore_liver_3fr_combo.cu",
}
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libbdoracle.so")
REF_SO = os.path.join(REF_OUT, "libbdref.so")

CXX = os.environ.get("CXX", "g++")
# -ffp-contract=off: no FMA contraction, so results agree between x86 and Arm hosts
COMMON = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "bd_oracle.cpp"), os.path.join(HERE, "..", "include", "bubbledyn.h")]
    if force or not _newer(ORACLE_SO, srcs):
        _run([CXX] + COMMON + ["-o", ORACLE_SO, srcs[0]])
    return ORACLE_SO


def extract_reference():
    """Write the lines before `int main()` of each reference file into _ref/src."""
    src_dir = os.path.join(REF_OUT, "src")
    os.makedirs(src_dir, exist_ok=True)
    for key, name in REF_FILES.items():
        path = os.path.join(REF_DIR, name)
        with open(path, "r", encoding="utf-8", errors="replace") as f:
            lines = f.readlines()
        cut = next(i for i, l in enumerate(lines) if l.startswith("int main()"))
        with open(os.path.join(src_dir, "%s_kernels.inc" % key), "w") as f:
            f.writelines(lines[:cut])


def extract_T_trajectory():
    """The spiral loop of the heat program (T:114-173 parameters, T:323-410 loop)
    as a function body: the kernel launch becomes a recorder of the per-step
    shift, the device synchronisation a no-op, and one brace closes the loop."""
    path = os.path.join(REF_DIR, REF_FILES["T"])
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        lines = f.readlines()
    body = lines[113:173] + lines[322:410]
    out = []
    for l in body:
        if "Temperature_square <<<" in l:
            out.append("            BDREF_RECORD(shift_x, shift_y, lines);\n")
        elif "cudaDeviceSynchronize" in l:
            out.append("\n")
        else:
            out.append(l)
    out.append("    }\n")
    with open(os.path.join(REF_OUT, "src", "T_traj.inc"), "w") as f:
        f.writelines(out)


def have_reference_sources():
    return all(os.path.exists(os.path.join(REF_DIR, n)) for n in REF_FILES.values())


def extract_all():
    """Extract the reference sections (when the reference tree is present)."""
    if have_reference_sources():
        extract_reference()
        extract_T_trajectory()


def build_ref(force=False, extract=True):
    """Build oracle/_ref/libbdref.so; returns its path or None if no sources."""
    src_dir = os.path.join(REF_OUT, "src")
    if extract:
        extract_all()
    incs = [os.path.join(src_dir, "%s_kernels.inc" % k) for k in REF_FILES] + [os.path.join(src_dir, "T_traj.inc")]
    if not all(os.path.exists(p) for p in incs):
        return None
    harness = os.path.join(HERE, "ref_harness.cpp")
    deps = incs + [harness, os.path.join(HERE, "ref_stub.h")]
    if force or not _newer(REF_SO, deps):
        _run([CXX] + COMMON + ["-O2", "-I", os.path.join(HERE, "ref_include"), "-I", HERE,
                                "-o", REF_SO, harness])
    return REF_SO


REF_GPU_SO = os.path.join(REF_OUT, "libbdref_gpu.so")


def build_ref_gpu(force=False, extract=True):
    """Build oracle/_ref/libbdref_gpu.so: the reference's W and G kernel
    sections compiled by nvcc for sm_103a with the host loops of
    ref_gpu_harness.cu.  Returns its path, or None without the sections."""
    src_dir = os.path.join(REF_OUT, "src")
    if extract:
        extract_all()
    incs = [os.path.join(src_dir, "%s_kernels.inc" % k) for k in ("W", "G")]
    if not all(os.path.exists(p) for p in incs):
        return None
    harness = os.path.join(HERE, "ref_gpu_harness.cu")
    if force or not _newer(REF_GPU_SO, incs + [harness]):
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
              "-Xcompiler", "-fPIC", "-diag-suppress", "177,550", "-I", HERE, "-o", REF_GPU_SO, harness])
    return REF_GPU_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_gpu(force="--force" in sys.argv))
