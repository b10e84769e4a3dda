"""Build the sm_103a shared library in-tree: eulersf_gb300/_lib/libeulersf_gb300.so.

Three translation units, compiled in parallel:
  esf_solver.cu  pressure stencil + PCR + solid block solver (FMA allowed)
  esf_step.cu    every other kernel and the C ABI, -fmad=false so flags, maps
                 and particle seeding keep the reference's non-FMA arithmetic
  esf_config.cpp the cfg reader
  esf_bake.cu    offline mass baking of a solid's rest mass from its mesh
  esf_contact.cu the rest-SDF (".svol") reader and triangle hash of
                 solid-solid contact
  esf_io.cpp     frame files (gz fields, OBJ); zlib is loaded at run time
  esf_serve.cpp  the multi-scene server (host threads, one stream per scene)
Host code is compiled with -ffp-contract=off for the same reason (the box's
aarch64 compiler would otherwise contract a*b+c).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libeulersf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return {
        "esf_solver.cu": ["-O3", "-lineinfo"],
        "esf_step.cu": ["-O3", "-lineinfo", "-fmad=false"],
        "esf_bake.cu": ["-O3", "-lineinfo"],
        "esf_contact.cu": ["-O2"],
        "esf_config.cpp": ["-O2"],
        "esf_io.cpp": ["-O2"],
        "esf_serve.cpp": ["-O2"],
    }


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "eulersf.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC]
    objs = []

    def one(item):
        src, flags = item
        obj = os.path.join(OUT, src + f".{os.getpid()}.o")
        cmd = [nvcc, "-c", os.path.join(CSRC, src), "-o", obj] + common + flags
        if src.endswith(".cpp"):
            cmd = [nvcc, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj, "-std=c++17",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-O2"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=7) as ex:
        objs = list(ex.map(one, _sources().items()))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    for o in objs:
        try:
            os.remove(o)
        except OSError:
            pass
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
