"""Builds the in-tree CUDA library ``libplenoxels_gb300.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit compiles in its own ``nvcc`` process (in parallel),
then one ``nvcc -shared`` link produces the library next to this file. Objects are
rebuilt only when a source or header is newer than them. No torch headers are involved:
the library exposes a plain C ABI (``include/plenoxels_gb300.h``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libplenoxels_gb300.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    # host-side fp32 arithmetic (splat camera constants) must round op by op on Arm too
    "-Xcompiler", "-ffp-contract=off",
    # IEEE division and square root, no flush to zero. FMA contraction stays on for the
    # compositing and gradient arithmetic; the index path (positions, normalisation,
    # rounding) is written with __fmul_rn/__fadd_rn/__fdiv_rn intrinsics, which nvcc never
    # contracts, so it rounds op by op as the reference's CPU arithmetic does
    "-fmad=true", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    f"-I{INCLUDE}", f"-I{CSRC}",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build plenoxels_gb300")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, jobs: int | None = None,
          extra_flags: list[str] | None = None, lib_path: str | None = None,
          build_dir: str | None = None) -> str:
    """Compiles and links the library; returns its path. extra_flags (e.g. -D tuning
    knobs of the kernels), lib_path and build_dir make an alternative build beside the
    default one (load it with PLENOXELS_GB300_LIB=<lib_path>)."""
    nvcc = _nvcc()
    bdir = build_dir or BUILD_DIR
    out = lib_path or LIB_PATH
    flags = NVCC_FLAGS + list(extra_flags or [])
    os.makedirs(bdir, exist_ok=True)
    headers = _headers()
    jobs_todo = []
    objects = []
    for src in _sources():
        obj = os.path.join(bdir, os.path.basename(src)[:-3] + ".o")
        objects.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs_todo.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stderr}")
        return res.stderr

    if jobs_todo:
        n = jobs or min(len(jobs_todo), os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=n) as ex:
            for msg in ex.map(compile_one, jobs_todo):
                if verbose and msg:
                    print(msg, file=sys.stderr)
    if force or jobs_todo or _stale(out, objects):
        tmp = out + ".tmp"
        cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", tmp] + objects + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
        os.replace(tmp, out)
    if lib_path is None:
        _build_probes(nvcc, verbose)
    return out


PROBES_DIR = os.path.join(PKG_DIR, "probes")
PROBES_LIB = os.path.join(PROBES_DIR, "libpgb_probes.so")


def _build_probes(nvcc: str, verbose: bool) -> str:
    """The measurement helper libpgb_probes.so (probes/probe.cu), its own small library."""
    src = os.path.join(PROBES_DIR, "probe.cu")
    deps = [src, os.path.join(PROBES_DIR, "pgb_probes.h")] + _headers()
    if not _stale(PROBES_LIB, deps):
        return PROBES_LIB
    tmp = PROBES_LIB + ".tmp"
    cmd = [nvcc] + NVCC_FLAGS + [f"-I{PROBES_DIR}", "-shared", src, "-o", tmp,
                                 "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"probe library build failed:\n{res.stderr}")
    os.replace(tmp, PROBES_LIB)
    return PROBES_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
