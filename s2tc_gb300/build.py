"""Build recipe for libs2tc_gb300.so (and the CPU checkers under oracle/).

Compiles every CUDA translation unit for sm_103a with nvcc, in parallel, and
links them with the host C ABI into ``s2tc_gb300/_lib/libs2tc_gb300.so``.  The
encoder translation unit is compiled once per colour-distance metric.
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
LIB_DIR = PKG / "_lib"
OBJ_DIR = LIB_DIR / "obj"
LIB_PATH = LIB_DIR / "libs2tc_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no float multiply-add contraction anywhere (the NORMALMAP and
# SRGB_MIXED metrics must round every float operation like the reference).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O2",
              "-I" + str(CSRC), "-I" + str(ROOT / "include")]
N_METRICS = 8


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _units():
    """(source, object, extra flags) for every translation unit."""
    units = []
    for m in range(N_METRICS):
        units.append((CSRC / "encode.cu", OBJ_DIR / f"encode_m{m}.o", [f"-DS2TC_METRIC={m}"]))
    for name in ("dither.cu", "dither_fs.cu", "noalloc.cu", "tools.cu", "rand_glibc.cu"):
        units.append((CSRC / name, OBJ_DIR / (Path(name).stem + ".o"), []))
    units.append((CSRC / "capi.cpp", OBJ_DIR / "capi.o", ["-x", "cu"]))
    units.append((CSRC / "server.cpp", OBJ_DIR / "server.o", ["-x", "cu"]))
    return units


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    # extra nvcc flags (e.g. -D tuning macros) force a rebuild when they change
    extra = os.environ.get("S2TC_NVCC_EXTRA", "").split()
    stamp = OBJ_DIR / "flags.txt"
    if not stamp.exists() or stamp.read_text() != " ".join(extra):
        force = True
        stamp.write_text(" ".join(extra))
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "s2tc_gb300.h"]
    jobs = []
    for src, obj, unit_flags in _units():
        if force or _stale(obj, [src, *headers]):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *unit_flags, *extra, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): cmd for cmd in jobs}
            for fut in cf.as_completed(futs):
                r = fut.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(" ".join(futs[fut]) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed")
    objs = [str(obj) for _, obj, _ in _units()]
    if force or jobs or not LIB_PATH.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB_PATH), *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    return LIB_PATH


# Where this recipe looks for the reference's sources (the build container's
# read-only checkout); S2TC_REFERENCE_DIR overrides it.  Machines without the
# sources (the GPU hosts) build only the restatement.
DEFAULT_REFERENCE_DIR = "/root/reference"


def reference_dir() -> Path | None:
    """The reference's source tree, or None where it is absent."""
    ref = Path(os.environ.get("S2TC_REFERENCE_DIR", DEFAULT_REFERENCE_DIR))
    return ref if (ref / "s2tc_algorithm.cpp").exists() else None


def build_oracle(verbose: bool = False) -> None:
    """The CPU restatement (always) and the reference's own encoder (only where
    its sources are present)."""
    oracle = ROOT / "oracle"
    targets = ["oracle"]
    ref = reference_dir()
    if ref is not None:
        targets.append("ref")
    else:
        ref = Path(DEFAULT_REFERENCE_DIR)
    r = subprocess.run(["make", "-C", str(oracle), f"REF={ref}", *targets], capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed")


def build(verbose: bool = False, force: bool = False) -> Path:
    build_oracle(verbose)
    return build_library(verbose, force)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB_PATH)
