"""Builds the engine's CUDA library in-tree: wavefiber3d_gb300/_build/libwavepo.so.

Every translation unit under csrc/ is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) in parallel, then linked into one
shared library with a C ABI (include/wavepo.h).  The drop-in command-line
drivers (cli/wavepo_cli.cpp: wavepo_sphere, wavepo_ellipsoid,
wavepo_ellipsoid_simple, wavepo_treepo) are linked against it into the same
folder.
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
LIB = BUILD / "libwavepo.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
           "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


CLI_SRC = PKG / "cli" / "wavepo_cli.cpp"
CLIS = {"wavepo_sphere": "SPHERE", "wavepo_ellipsoid": "ELLIPSOID", "wavepo_ellipsoid_simple": "ELLIPSOID_SIMPLE",
        "wavepo_treepo": "TREEPO"}


def _build_cli(name: str, define: str) -> Path:
    exe = BUILD / name
    cmd = [nvcc(), "-O2", "-std=c++17", f"-DWAVEPO_CLI_{define}", "-I", str(ROOT / "include"), str(CLI_SRC), "-o",
           str(exe), "-L", str(BUILD), "-lwavepo", "-Xlinker", "-rpath,$ORIGIN", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
    return exe


def build_cli(force: bool = False) -> list:
    """Links the drop-in drivers against libwavepo.so (after build())."""
    t = LIB.stat().st_mtime
    todo = [n for n in CLIS if force or not (BUILD / n).exists() or (BUILD / n).stat().st_mtime < max(
        t, CLI_SRC.stat().st_mtime, (ROOT / "include" / "wavepo.h").stat().st_mtime)]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        list(ex.map(lambda n: _build_cli(n, CLIS[n]), todo))
    return [BUILD / n for n in CLIS]


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    deps = srcs + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "wavepo.h"]
    if LIB.exists() and not force and not verbose_ptxas:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in deps):
            build_cli()
            return LIB
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = BUILD / "libwavepo.so.tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    tmp.replace(LIB)
    build_cli(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
