"""Build the CUDA library ``libpnepma_gb300.so`` in-tree (``pnepma_gb300/_build``).

Every translation unit is compiled by nvcc for sm_103a only; the per-order units compile in
parallel.  The stencil header is regenerated first from the closed-form coupling blocks.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

from . import codegen

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpnepma_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include", "pnepma.h")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources():
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(CSRC, "generated", f) for f in os.listdir(os.path.join(CSRC, "generated"))]
    return headers + [INCLUDE]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(args):
    src, obj, defines, extra = args
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + defines + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False, out: str | None = None,
          defines=()) -> str:
    """Compile every unit for sm_103a and link the library.  `out` and `defines` build a variant
    (e.g. another occupancy bound) into another directory; the default is the in-tree library."""
    out_dir = out or OUT
    lib_path = os.path.join(out_dir, os.path.basename(LIB))
    os.makedirs(out_dir, exist_ok=True)
    codegen.write_header()
    deps = _sources()
    jobs = []
    objs = []
    extra = (["-Xptxas", "-v"] if ptxas_verbose else []) + list(defines)
    capi = os.path.join(CSRC, "pn_capi.cu")
    o = os.path.join(out_dir, "pn_capi.o")
    objs.append(o)
    if force or _stale(o, deps + [capi]):
        jobs.append((capi, o, [], extra))
    # the material unit rounds every product and sum separately, as the reference's Julia code does
    unit_flags = {"pn_material": ["-fmad=false"]}
    for unit in ("pn_batch", "pn_noalloc", "pn_server", "pn_selftest", "pn_material"):
        src = os.path.join(CSRC, unit + ".cu")
        o = os.path.join(out_dir, unit + ".o")
        objs.append(o)
        if force or _stale(o, deps + [src]):
            jobs.append((src, o, [], extra + unit_flags.get(unit, [])))
    for unit in ("pn_order", "pn_order_batch"):
        src = os.path.join(CSRC, unit + ".cu")
        for N in codegen.ORDERS:
            o = os.path.join(out_dir, f"{unit}_{N}.o")
            objs.append(o)
            if force or _stale(o, deps + [src]):
                jobs.append((src, o, [f"-DPN_ORDER={N}"], extra))
    # longest units first so the parallel build finishes sooner
    jobs.sort(key=lambda j: -int(next((d.split("=")[1] for d in j[2] if d.startswith("-DPN_ORDER=")), "0")))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 1))
        with ThreadPoolExecutor(workers) as ex:
            for log in ex.map(_compile, jobs):
                if verbose and log:
                    print(log, file=sys.stderr)
    if force or jobs or _stale(lib_path, objs):
        tmp = lib_path + f".tmp{os.getpid()}"
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_verbose="-v" in sys.argv))
