"""Build libcvl_gb300.so (the CUDA library) and the CPU oracle in place.

The library is plain nvcc output for sm_103a: every ``csrc/*.cu`` file is
compiled to an object in parallel and linked into one shared library next to
this file.  No PyTorch extension machinery is involved; the library exports
the C ABI declared in ``include/cvl_gb300.h``.
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
BUILD = PKG / "_build"
LIB = PKG / "libcvl_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", str(CSRC), "-I", str(ROOT / "include"),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    return cand


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def tuning_defines() -> list[str]:
    """-D flags for the kernels' tuning macros (GCVL_RK_ITEMS, GCVL_RING_MINB,
    ...) from GCVL_TUNE="NAME=VALUE ...": for timing other tile and
    occupancy choices than the defaults in the sources."""
    return [f"-D{x}" for x in os.environ.get("GCVL_TUNE", "").split() if x.startswith("GCVL_")]


def build_library(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    tune = tuning_defines()
    stamp = BUILD / "tuning"
    if (stamp.read_text() if stamp.exists() else "") != " ".join(tune):
        force = True  # objects built with other tuning macros
    objs = []
    jobs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers, Path(__file__)]):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *tune, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    workers = min(len(jobs), os.cpu_count() or 4) or 1
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-ldl"]
        run(cmd)
    stamp.write_text(" ".join(tune))
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) and, where the reference
    tree is mounted, the reference's own serial CVL into oracle/_ref."""
    odir = ROOT / "oracle"
    r = subprocess.run(["make", "-s", "-C", str(odir)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    # the oracle's Makefile knows where the reference tree is mounted
    # (GCVL_REFERENCE overrides) and skips the build where it is not
    args = ["make", "-s", "-C", str(odir), "ref"]
    if os.environ.get("GCVL_REFERENCE"):
        args.append(f"REF={Path(os.environ['GCVL_REFERENCE']) / 'nesl'}")
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0 and verbose:
        print("reference serial CVL not built:", r.stderr, file=sys.stderr)
    return odir / "_build" / "libcvl_oracle.so"


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build_library(verbose=v, force="-f" in sys.argv))
    print(build_oracle(verbose=v))
