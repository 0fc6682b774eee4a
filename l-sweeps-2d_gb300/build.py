"""Build liblsweeps_gb300.so in-tree: every translation unit of csrc/ (the
kernels and the C ABI) and host/ (the C++ classes of the reference's plugin
API) compiled for sm_103a in parallel with nvcc and linked with the static
CUDA runtime, plus the driver executable lsweeps_gb300_main."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
HOST = HERE / "host"
MAIN = HERE / "lsweeps" / "lsweeps_gb300_main"
OUT_DIR = HERE / "_build"
LIB = HERE / "lsweeps" / "liblsweeps_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _flags(verbose_ptxas: bool) -> list[str]:
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}", f"-I{CSRC}"] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: Path, verbose_ptxas: bool) -> tuple[Path, str]:
    obj = OUT_DIR / ((src.parent.name + "_") + src.stem + ".o")
    cmd = [nvcc(), "-c", str(src), "-o", str(obj)] + _flags(verbose_ptxas)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose_ptxas: bool = False, force: bool = False) -> Path:
    srcs = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    srcs += [HOST / "host.cpp", HOST / "input.cpp"]
    deps = srcs + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "lsweeps.h",
                                                                          ROOT / "include" / "lsweeps_host.hpp",
                                                                          HOST / "main.cpp"]
    if LIB.exists() and MAIN.exists() and not force and not verbose_ptxas:
        t = min(LIB.stat().st_mtime, MAIN.stat().st_mtime)
        if all(d.stat().st_mtime <= t for d in deps):
            return LIB
    OUT_DIR.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if verbose_ptxas:
        for _, log in res:
            sys.stderr.write(log)
    objs = [str(o) for o, _ in res]
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + objs + ARCH + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the reference's driver (main.cpp) over the library
    tmpm = MAIN.with_suffix(".tmp")
    cmd = [nvcc(), str(HOST / "main.cpp"), "-o", str(tmpm), "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
           f"-L{LIB.parent}", "-llsweeps_gb300", "-Xlinker", "-rpath=$ORIGIN"] + ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmpm, MAIN)
    return LIB


if __name__ == "__main__":
    p = build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
