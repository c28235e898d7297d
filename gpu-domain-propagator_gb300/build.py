"""Build the native libraries of the GB300 domain propagator in-tree.

    libgdp_gb300.so  -- CUDA kernels (sm_103a) + host driver + C-ABI (include/*.h)
    libgdpgen.so     -- seeded synthetic MIP generators (host C++)

Both land in gpu-domain-propagator_gb300/lib/. `--phase-timers` builds, beside
them, libgdp_gb300_timers.so: the same library compiled with
-DGDP_PHASE_TIMERS, whose megakernel records per-round phase times
(gdp_phase_timers_read; phase_split.py prints them). It is slower by the
timers' atomics and is never loaded by default. `--build-timers` builds
libgdp_gb300_buildtimers.so (-DGDP_BUILD_TIMERS): every context build prints
the times of its milestones to stderr. Translation units compile in
parallel; one -gencode (compute_103a / sm_103a) keeps the build to about a
minute.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
OBJ = PKG / "lib" / "obj"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["gdp_round.cu", "gdp_context.cu", "gdp_capi.cu", "gdp_noalloc.cu", "gdp_layout.cu", "gdp_batch.cu",
                "gdp_batch_host.cu", "gdp_mlp.cu", "gdp_learned.cu", "gdp_tune.cu", "gdp_mps.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgdp_gb300.so")


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, cwd=str(CSRC), capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, flush=True)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def nvcc_flags(extra: list[str] | None = None) -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
        "-Xcompiler", "-fPIC,-fopenmp,-O3,-fvisibility=hidden",
        f"-I{INCLUDE}", f"-I{CSRC}",
    ] + (extra or [])


def build(verbose: bool = False, force: bool = False, phase_timers: bool = False,
          build_timers: bool = False) -> dict[str, Path]:
    tag = ("_timers" if phase_timers else "") + ("_buildtimers" if build_timers else "")
    obj_dir = OBJ.with_name(OBJ.name + tag)
    defines = (["-DGDP_PHASE_TIMERS"] if phase_timers else []) + (["-DGDP_BUILD_TIMERS"] if build_timers else [])
    LIB.mkdir(parents=True, exist_ok=True)
    obj_dir.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        o = obj_dir / (Path(src).stem + ".o")
        objs.append(o)
        if force or _stale(o, [CSRC / src] + headers):
            jobs.append([nvcc, *nvcc_flags(defines), "-c", str(CSRC / src), "-o", str(o)])
    gen_so = LIB / "libgdpgen.so"
    gen_job = None
    if force or _stale(gen_so, [CSRC / "gdp_gen.cpp", CSRC / "gdp_gen.h"]):
        gen_job = ["g++", "-O3", "-fPIC", "-fopenmp", "-std=c++17", "-shared", f"-I{CSRC}",
                   str(CSRC / "gdp_gen.cpp"), "-o", str(gen_so)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        futs = [ex.submit(_run, j, verbose) for j in jobs]
        if gen_job:
            futs.append(ex.submit(_run, gen_job, verbose))
        for f in futs:
            f.result()
    so = LIB / f"libgdp_gb300{tag}.so"
    if force or jobs or not so.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(so), *map(str, objs), "-Xcompiler", "-fopenmp",
              "-lgomp"], verbose)
    return {"gdp": so, "gen": gen_so}


if __name__ == "__main__":
    out = build(verbose="-v" in sys.argv, force="-f" in sys.argv, phase_timers="--phase-timers" in sys.argv,
                build_timers="--build-timers" in sys.argv)
    for k, v in out.items():
        print(k, v)
