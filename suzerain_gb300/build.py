"""Build libsuzerain_gb300.so in-tree: nvcc for sm_103a, one -gencode.

Translation units compile in parallel (one worker per host core), then link with the static CUDA
runtime, so the library carries no dependency on torch's runtime copy.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libsuzerain_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build")


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) +
                  glob.glob(os.path.join(CSRC, "*.cpp")))


# gbtrf_blk_inst.cu is compiled once per (precision, panel width, warp
# family): each object holds 8 of the 192 blocked-factor kernels.
BLK_INST = "gbtrf_blk_inst.cu"
BLK_VARIANTS = [(p, nb, fam) for nb in (16, 8, 4) for p in ("z", "c")
                for fam in (0, 1, 2, 4)]
# and once per bandwidth of the compile-time complex64 instances
BLK_SPEC_BANDS = (24, 34)


def jobs() -> list[tuple[str, str, list[str]]]:
    """(source, object stem, extra flags) per object, the heaviest first."""
    out = []
    for src in sources():
        if os.path.basename(src) == BLK_INST:
            for p, nb, fam in BLK_VARIANTS:
                r = "double" if p == "z" else "float"
                out.append((src, f"gbtrf_blk_{p}{nb}_f{fam}",
                            [f"-DSGB_BLK_R={r}", f"-DSGB_BLK_NB={nb}",
                             f"-DSGB_BLK_FAM={fam}"]))
            for kb in BLK_SPEC_BANDS:
                out.append((src, f"gbtrf_blk_spec{kb}", [f"-DSGB_BLK_SPEC={kb}"]))
        else:
            out.append((src, os.path.basename(src), []))
    return out


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + _headers()
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "suzerain_gb300.h"), __file__]


def _compile(job: tuple[str, str, list[str]], nvcc: str, debug: bool,
             force: bool = False) -> str:
    src, stem, defs = job
    obj = os.path.join(OBJ_DIR, stem + (".dbg.o" if debug else ".o"))
    if not force and os.path.exists(obj):
        # an object newer than its source and every header is current
        t = os.path.getmtime(obj)
        if all(os.path.getmtime(d) < t for d in [src] + _headers()):
            return obj
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler",
               "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr", *inc,
               *defs, "-c", src, "-o", obj]
        if debug:
            cmd.insert(1, "-DSGB_DEBUG_BOUNDS")
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
               "-Wall", *inc, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n"
                           f"{r.stderr}")
    return obj


def build(force: bool = False, debug: bool = False, verbose: bool = False
          ) -> str:
    """Compile every CUDA/C++ source and link the shared library."""
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJ_DIR, exist_ok=True)
    js = jobs()
    workers = max(1, min(len(js), os.cpu_count() or 8))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda j: _compile(j, nvcc, debug, force), js))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart=static", "-o", tmp, *objs,
           "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
