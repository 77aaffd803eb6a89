"""Builds libHYPRE_gb300.so in-tree: the C host library (gcc) and the sm_103a
kernels (nvcc), linked with the CUDA runtime.  No torch involvement.

    python -m hypre_gb300.build        (or __graft_entry__.build())
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libHYPRE_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, ptxas_info=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", os.path.join(cuda, "include")]
    jobs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        if f.endswith(".cu"):
            # the setup kernels reproduce the reference's serial rounding: no FMA contraction
            fmad = "false" if f in ("gb_setup.cu", "gb_agg.cu", "gb_hgs.cu", "gb_multipass.cu") else "true"
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=" + fmad, "-Xcompiler", "-fPIC",
                                   "-c", src, "-o", obj] + inc
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append((cmd, obj))
        elif f.endswith(".c"):
            cmd = ["gcc", "-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-function", "-ffp-contract=off",
                   "-c", src, "-o", obj] + inc
            if f == "gb_ij.c":
                cmd.insert(1, "-fopenmp")   # host passes over the rows of large IJ puts
            jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    objs = [o for _, o in jobs]
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lgomp", "-lrt", "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
