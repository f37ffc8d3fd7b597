"""Builds the parent_gb300 native code in-tree.

Outputs (all git-ignored):
  parent_gb300/lib/libparent_gb300.so   the C-ABI library (CUDA for sm_103a + host C++)
  parent_gb300/bin/*_gb300             the command-line drop-ins
  parent_gb300/_build/*.o              objects (rebuilt only when a source or header changed)

Only nvcc (one -gencode, arch=compute_103a,code=sm_103a) and g++ are used; the
translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CLI = PKG / "cli"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
BINDIR = PKG / "bin"
LIB = LIBDIR / "libparent_gb300.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags. pg_prep decides bin indices, so it must not
# contract a*b+c into FMA anywhere (bit-exact with the reference's FP64).
CU_SOURCES = {
    "pg_api.cu": [],
    "pg_prep.cu": ["--fmad=false"],
    "pg_pairs_hist.cu": [],
    "pg_pairs_hist32.cu": [],
    "pg_pairs_onehot.cu": [],
    "pg_mist.cu": [],
    "pg_synth.cu": [],
    "pg_noalloc.cu": [],
    "pg_ingest.cu": [],
    "pg_batconv.cu": ["--fmad=false"],
    "pg_mie.cu": [],
    "pg_autotune.cu": [],
}
CPP_SOURCES = ["pg_io.cpp", "pg_io_compat.cpp"]
CLIS = ["PARENT_gb300", "get_PAR_MIST_gb300", "get_PAR_MIE_gb300", "get_PAR_info_gb300"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _newer(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} ... {cmd[-1]}")


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles the library and CLIs if anything is out of date; returns the .so path."""
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    BINDIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + [INCLUDE / "parent_gb300.h", INCLUDE / "parent_gb300_io.h"]
    steps = []
    objs = []
    for src, extra in CU_SOURCES.items():
        s = CSRC / src
        if not s.exists():
            continue
        o = BUILD / (src + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            steps.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                          "-Xcompiler", "-fvisibility=hidden", "-I", str(INCLUDE), *extra,
                          "-c", str(s), "-o", str(o)])
    for src in CPP_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            steps.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall",
                          "-I", str(INCLUDE), "-I", str(home / "include"), "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for cmd in steps:
            if verbose:
                print(" ".join(cmd))
        list(ex.map(_run, steps))
    if steps or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(LIB),
              "-lpthread"])
    cli_steps = []
    for name in CLIS:
        src = CLI / f"{name}.cpp"
        out = BINDIR / name
        if not _newer(out, [src, CLI / "common.h", LIB, INCLUDE / "parent_gb300.h"]):
            cli_steps.append(["g++", "-O2", "-std=c++17", "-Wall", "-I", str(INCLUDE), str(src),
                              "-L", str(LIBDIR), "-lparent_gb300", "-Wl,-rpath,$ORIGIN/../lib",
                              "-o", str(out)])
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, cli_steps))
    return LIB


def build_oracle() -> Path:
    """Compiles the oracle (test infrastructure) and, when the reference
    sources are present on this machine, the reference programs it is pinned
    against."""
    oracle = ROOT / "oracle"
    _run(["make", "-s", "-C", str(oracle)])
    # the recipe's REF_ROOT (or PG_REFERENCE_ROOT) says where the reference sources are
    r = subprocess.run(["make", "-s", "-C", str(oracle), "print-ref-root"], capture_output=True, text=True)
    ref_root = r.stdout.strip()
    if ref_root and (Path(ref_root) / "src" / "PARENT" / "PARENT.cpp").exists():
        _run(["make", "-s", "-C", str(oracle), "ref", "-j4"])
    return oracle / "liboracle.so"


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(build_oracle())
