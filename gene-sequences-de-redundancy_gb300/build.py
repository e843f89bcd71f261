"""Builds the native parts in-tree: libgsdr.so (CUDA kernels for sm_103a +
C ABI), the `cluster` executable, and libgsdr_synth.so (workload generator).

    python gene-sequences-de-redundancy_gb300/build.py

Each translation unit compiles in its own process; outputs go to
gene-sequences-de-redundancy_gb300/_build/.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INC = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = ["prep.cu", "rounds.cu", "api.cu", "noalloc.cu", "server.cu", "devparse.cu", "devmem.cu",
      "autotune.cu"]
CPP = ["fasta.cpp"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(INC, f) for f in os.listdir(INC)]
    jobs = []
    objs = []
    for f in CU:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if newer(obj, [src] + headers):
            jobs.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xptxas", "-v",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INC, "-I", SRC,
                         "-c", src, "-o", obj])
    for f in CPP:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if newer(obj, [src] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", INC, "-I", SRC, "-c", src, "-o", obj])
    synth_src = os.path.join(SRC, "synth.cpp")
    synth_so = os.path.join(OUT, "libgsdr_synth.so")
    if newer(synth_so, [synth_src] + headers):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                     "-ffp-contract=off", "-I", INC, synth_src, "-o", synth_so])
    logs = []
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(run, jobs):
            logs.append(out)
    lib = os.path.join(OUT, "libgsdr.so")
    if newer(lib, objs):
        run([nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-Xcompiler", "-fPIC"])
    cli = os.path.join(OUT, "cluster")
    cli_src = os.path.join(SRC, "cli.cpp")
    if newer(cli, [cli_src, lib]):
        run(["g++", "-O2", "-std=c++17", "-I", INC, cli_src, "-o", cli, "-L", OUT, "-lgsdr",
             "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", OUT)
