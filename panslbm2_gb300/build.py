"""Build the CUDA library in-tree: panslbm2_gb300/libpanslbm_gb300.so (sm_103a).

Translation units compile in parallel. The FP64 instantiation units are compiled with
-fmad=false so their arithmetic matches the reference's scalar CPU path operation for
operation; every other unit keeps FMA contraction (the throughput path), and the FP32 / 16-bit
instantiation units use the fast single-precision division (-prec-div=false, within 2 ulp).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpanslbm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-Xcompiler", "-Wall,-Wno-unused-function", "-I", CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu"):
            out.append(os.path.join(CSRC, f))
    return out


def deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(HERE, "..", "include", "panslbm_gb300.h")]


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    flags = list(COMMON)
    if "_f64" in os.path.basename(src):
        flags += ["-fmad=false"]
    elif "inst_" in os.path.basename(src):
        flags += ["-prec-div=false"]
    if verbose_ptxas:
        flags += ["-Xptxas", "-v"]
    cmd = [nvcc()] + ARCH + flags + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, p.stdout, p.stderr))
    return obj, p.stderr


def build(force=False, jobs=None, verbose_ptxas=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    newest_dep = max(os.path.getmtime(d) for d in deps())
    todo = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        if force or verbose_ptxas or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_dep):
            todo.append(s)
    logs = {}
    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for src, (obj, log) in zip(todo, ex.map(lambda s: _compile(s, verbose_ptxas), todo)):
                logs[src] = log
    objs = [os.path.join(OBJ, os.path.basename(s) + ".o") for s in srcs]
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(force="-f" in sys.argv, verbose_ptxas="-v" in sys.argv)
    for k, v in logs.items():
        if v.strip():
            print("==", os.path.basename(k))
            print(v)
    print(lib)
