"""Build the CUDA library libphyskit_gb300.so in-tree (physkit_gb300/_lib/).

nvcc for sm_103a only, one -gencode, translation units compiled in parallel:
  pk_engine_f64.cu  FP64 parity engine, -fmad=false (every multiply and add rounds as written)
  pk_engine_f32.cu  FP32 precision engine (fused multiply-adds allowed)
  pk_capi.cu        the C ABI of include/physkit_gb300.h (host code, -ffp-contract=off)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libphyskit_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
UNITS = {
    "pk_engine_f64.cu": ["-fmad=false"],
    "pk_engine_f32.cu": ["-fmad=true"],
    "pk_capi.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build physkit_gb300")


def _deps():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(ROOT, "include", "physkit_gb300.h"),
                                                            os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    objs = []

    def compile_one(name):
        obj = os.path.join(OUT, name.replace(".cu", ".o"))
        extra = os.environ.get("PK_NVCC_FLAGS", "").split()  # optional extra nvcc flags
        cmd = [nv, *ARCH, *COMMON, *UNITS[name], *extra, "-c", os.path.join(SRC, name), "-o", obj]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for obj, err in ex.map(compile_one, list(UNITS)):
            objs.append(obj)
            if verbose and err:
                print(err, file=sys.stderr)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv))
