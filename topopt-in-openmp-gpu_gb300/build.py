"""Builds libtopopt_gb300.so in-tree with nvcc for sm_103a (GB300).

    python topopt-in-openmp-gpu_gb300/build.py [-v] [--ptxas]

Translation units compile in parallel into _build/ and link into
topopt-in-openmp-gpu_gb300/libtopopt_gb300.so (and the reference-signature
wrapper libraries next to it). No cmake; one -gencode.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
INC = os.path.join(ROOT, "include")
NVCC = os.environ.get("NVCC", "nvcc")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INC, "-I", CSRC]
LIB = os.path.join(PKG, "libtopopt_gb300.so")


def _compile(src, verbose, ptxas):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [NVCC] + ARCH + FLAGS + ["-c", src, "-o", obj]
    if ptxas and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(verbose=False, ptxas=False):
    os.makedirs(BUILD, exist_ok=True)
    core = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")) and not f.startswith("tp_ref_api"))
    objs = []
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for src, obj, rc, out in ex.map(lambda s: _compile(s, verbose, ptxas), core):
            if out.strip():
                logs.append(out)
            if rc != 0:
                sys.stderr.write(out)
                raise RuntimeError("nvcc failed on " + src)
            objs.append(obj)
    cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    # reference-signature drop-in wrappers (float as shipped, double oracle form)
    ref_src = os.path.join(CSRC, "tp_ref_api.cpp")
    if os.path.exists(ref_src):
        for flav, define in (("32", "TP_REF_FLOAT=1"), ("64", "TP_REF_FLOAT=0")):
            out = os.path.join(PKG, "libtopopt_ref%s.so" % flav)
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-D" + define, "-I", INC,
                   "-I", CSRC, "-I", os.path.join(CUDA, "include"), ref_src, "-o", out, "-L" + PKG,
                   "-ltopopt_gb300", "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("ref wrapper build failed")
    if ptxas or verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas="--ptxas" in sys.argv))
