"""Builds libtis_gpu.so in-tree (16s-central-folding_gb300/_build/) with nvcc for sm_103a."""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libtis_gpu.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["tis_kernels.cu", "tis_engine.cu", "tis_system.cpp", "tis_loader.cpp", "tis_noalloc.cu", "tis_output.cpp",
           "tis_adjoint.cu", "tis_autotune.cpp", "tis_density.cu"]
RUN = os.path.join(OUT, "tis_run")  # the command-line program (csrc/tis_run.cpp) over the library


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I", os.path.join(PKG, "..", "include")]


# The step's kernels are compiled without implicit multiply-add contraction: the
# same device functions run in the separate kernels and in the persistent fused
# kernel, and contraction chosen per surrounding code would round them
# differently; explicit fma() calls stay fused.
NO_FMAD = {"tis_kernels.cu"}


def _compile(src):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    inp = os.path.join(CSRC, src)
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    extra = ["-fmad=false"] if src in NO_FMAD else []
    cmd = [NVCC, *_flags(), *extra, *lang, "-c", inp, "-o", obj]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return obj


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES + ["tis_run.cpp"]] + \
        [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    srcs.append(os.path.join(PKG, "..", "include", "tis_gpu.h"))
    if not force and os.path.exists(LIB) and os.path.exists(RUN) and \
            min(os.path.getmtime(LIB), os.path.getmtime(RUN)) > max(os.path.getmtime(s) for s in srcs):
        return LIB
    try:
        with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
            objs = list(ex.map(_compile, SOURCES))
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(NVCC))), "lib64")
        cmd = [NVCC, "-std=c++17", "-O2", "-I", os.path.join(PKG, "..", "include"), "-x", "c++",
               os.path.join(CSRC, "tis_run.cpp"), "-o", RUN, "-L", OUT, "-ltis_gpu",
               "-Xlinker", "-rpath,$ORIGIN:" + cuda_lib]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    except subprocess.CalledProcessError as e:
        raise RuntimeError(f"building libtis_gpu.so failed:\n{' '.join(e.cmd)}\n{e.stdout}\n{e.stderr}") from None
    if verbose:
        print("built", LIB)
    return LIB
