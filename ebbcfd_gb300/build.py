"""Build the in-tree shared library ebbcfd_gb300/_build/libebbgb300.so for sm_103a.

nvcc compiles the CUDA translation units (FP64 kernels with -fmad=false so that no
multiply-add is fused), g++ the host C++ (-ffp-contract=off for the same reason:
the FP64 geometry precompute must round like the reference's); everything links
into one shared library with a static CUDA runtime.  Compiles run in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libebbgb300.so")
CLI = os.path.join(OUT, "ebb-solve")
RECON = os.path.join(OUT, "ebb-reconstruct")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = {
    "k_fp64.cu": ["-fmad=false"],
    "k_split.cu": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
    "k_df.cu": ["-fmad=true", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
    "flux_noalloc.cu": ["-fmad=false"],
}
# extra -D overrides of the tuned launch shapes (csrc/tuned.h), set by the autotuner's variants
DEFINES = []
CPP = ["solver.cpp", "arena.cpp", "server.cpp", "reconstruct.cpp", "host_mesh.cpp", "host_config.cpp", "host_io.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ebbcfd_gb300")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _sources():
    srcs = [os.path.join(CSRC, f) for f in list(CU) + CPP + ["ebb_solve.cpp", "ebb_reconstruct.cpp"]]
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".hpp", ".cuh"))]
    hdr.append(os.path.join(os.path.dirname(HERE), "include", "ebb_gb300.h"))
    return srcs, hdr


def up_to_date():
    if not all(os.path.exists(f) for f in (LIB, CLI, RECON)):
        return False
    srcs, hdr = _sources()
    t = min(os.path.getmtime(f) for f in (LIB, CLI, RECON))
    return all(os.path.getmtime(f) <= t for f in srcs + hdr + [os.path.abspath(__file__)])


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for f, extra in CU.items():
        obj = os.path.join(OUT, f + ".o")
        jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
                    + extra + DEFINES + ["-c", os.path.join(CSRC, f), "-o", obj])
    for f in CPP:
        obj = os.path.join(OUT, f + ".o")
        jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                     "-I" + os.path.join(cuda, "include")] + DEFINES + ["-c", os.path.join(CSRC, f), "-o", obj])

    def run(cmd):
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        return cmd, p.returncode, p.stdout

    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        results = list(ex.map(run, jobs))
    logs = []
    for cmd, rc, out in results:
        logs.append(out)
        if rc != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), out))
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    objs = [os.path.join(OUT, f + ".o") for f in list(CU) + CPP]
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), p.stdout))
    os.replace(tmp, LIB)
    # the ebb-solve and ebb-reconstruct command-line drivers, linked against the library
    # (rpath $ORIGIN)
    for exe, src in ((CLI, "ebb_solve.cpp"), (RECON, "ebb_reconstruct.cpp")):
        tmp = exe + ".tmp%d" % os.getpid()
        cmd = ["g++", "-O2", "-std=c++17", "-o", tmp, os.path.join(CSRC, src), "-L" + OUT, "-lebbgb300",
               "-Wl,-rpath,$ORIGIN"]
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError("%s link failed: %s\n%s" % (os.path.basename(exe), " ".join(cmd), p.stdout))
        os.replace(tmp, exe)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
