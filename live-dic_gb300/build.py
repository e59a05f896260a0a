"""Build libgbdic.so (sm_103a) in-tree.

    python live-dic_gb300/build.py            # incremental
    python live-dic_gb300/build.py --force    # rebuild everything

Each .cu translation unit is compiled by nvcc in parallel, then linked into
live-dic_gb300/live_dic_gb300/libgbdic.so with the static CUDA runtime.
--fmad=false is part of the numerical contract of the kernels that are
bit-exact against the oracle (prefilter, IC-GN, outlier pass, pyramid,
seed transfer, temporal, ZNCC search, spatial seeds): a*b+c is fused only
where the source writes fmaf().  The units held to a tolerance instead
(reference preparation, Fourier initializer, the seed network's kernels)
compile with contraction on.
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
OUTPUT = ROOT / "live_dic_gb300" / "libgbdic.so"
INCLUDE = ROOT.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE)]
# Units whose results are checked against a tolerance, not bit for bit.
CONTRACTED = {"refprep", "refprep_rows", "fourier", "nn_ops", "nn_api", "tc_gemm", "solver_fast"}


def unit_flags(unit: Path) -> list[str]:
    # GBDIC_NVCC_DEFINES: extra -D tuning macros (e.g. GBDIC_FAST_MIN_BLOCKS), for sweeps
    extra = os.environ.get("GBDIC_NVCC_DEFINES", "").split()
    return ["--fmad=true" if unit.stem in CONTRACTED else "--fmad=false", *extra]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = Path("/usr/local/cuda/bin/nvcc")
    if candidate.exists():
        return str(candidate)
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgbdic.so")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    units = sorted(CSRC.glob("*.cu"))
    compiler = nvcc()
    jobs = []
    objects = []
    for unit in units:
        obj = BUILD / (unit.stem + ".o")
        objects.append(obj)
        cmd = [compiler, *ARCH, *FLAGS, *unit_flags(unit), "-c", str(unit), "-o", str(obj)]
        stamp = obj.with_suffix(".cmd")
        same_cmd = stamp.exists() and stamp.read_text() == " ".join(cmd)
        if force or not same_cmd or _stale(obj, [unit, *headers]):
            jobs.append(cmd)

    def run(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{result.stdout}\n{result.stderr}")
        if "-c" in cmd:
            Path(cmd[-1]).with_suffix(".cmd").write_text(" ".join(cmd))

    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with ThreadPoolExecutor(max_workers=workers) as pool:
            list(pool.map(run, jobs))
    if force or jobs or _stale(OUTPUT, objects):
        link = [compiler, *ARCH, "-shared", "-o", str(OUTPUT), *map(str, objects)]
        run(link)
    return OUTPUT


if __name__ == "__main__":
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--force", action="store_true")
    parser.add_argument("--verbose", action="store_true")
    args = parser.parse_args()
    print(build(force=args.force, verbose=args.verbose))
