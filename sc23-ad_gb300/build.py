"""Build libsagb.so (host setup + sm_103a CUDA kernels + C ABI) in-tree.

    python sc23-ad_gb300/build.py            # -> sc23-ad_gb300/_build/libsagb.so

Host C++ is compiled without FP contraction: the AMG setup must reproduce the
reference's FP64 values bit for bit on x86 and on Arm.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsagb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SRC = ["host/amg_setup.cpp", "host/schedule.cpp", "host/generators.cpp", "host/features.cpp",
            "host/batch_setup.cpp"]
CUDA_SRC = ["cuda/spmv.cu", "cuda/trsv.cu", "cuda/amg.cu", "cuda/krylov.cu", "cuda/mlp.cu", "cuda/batch.cu", "cuda/batch_fp.cu",
            "cuda/rs_setup.cu", "capi.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    NV = nvcc()
    jobs = []
    objs = []
    for s in HOST_SRC:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        jobs.append(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-c",
                     os.path.join(SRC, s), "-o", o])
    for s in CUDA_SRC:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        cmd = [NV, *ARCH, "-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", os.path.join(SRC, s), "-o", o]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        logs = list(ex.map(_compile, jobs))
    if verbose or ptxas_info:
        for l in logs:
            if l:
                sys.stderr.write(l)
    _compile([NV, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lpthread", "-ldl", "-lrt"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
