"""Build recipe for libmsbfs.so (sm_103a kernels + C++ host runtime).

Compiles every translation unit under csrc/ in parallel with nvcc (one
-gencode, sm_103a only) and links an in-tree shared library at
webgpu_bfs_gb300/_lib/libmsbfs.so. Objects are rebuilt only when a source or
header is newer than them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
LIB = LIBDIR / "libmsbfs.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(src: Path, obj: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def _compile(src: Path, obj: Path, verbose: bool, defines=()) -> None:
    dflags = [f"-D{d}" for d in defines]
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *dflags, "-c", str(src), "-o", str(obj)]
        if os.environ.get("MSBFS_PTXAS_VERBOSE"):
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++", *CXX_FLAGS, *dflags, f"-I{_cuda_include()}", "-c", str(src), "-o",
               str(obj)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)


def build_native(verbose: bool = False, force: bool = False, defines=(),
                 out_dir: Path | None = None) -> Path:
    """Builds (if needed) and returns the path of libmsbfs.so.

    `defines` are tuning macros (e.g. MSBFS_PULL_CH=8) and `out_dir` an
    alternative output folder, for building tuning variants side by side."""
    libdir = Path(out_dir) if out_dir else LIBDIR
    objdir = libdir / "obj"
    lib = libdir / "libmsbfs.so"
    objdir.mkdir(parents=True, exist_ok=True)
    # Objects built on another host architecture are never reused.
    stamp = libdir / "arch.txt"
    arch = platform.machine()
    if not stamp.exists() or stamp.read_text().strip() != arch:
        force = True
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    objs = []
    for src in sources:
        obj = objdir / (src.name + ".o")
        objs.append(obj)
        if force or _stale(src, obj, newest_header):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, verbose, defines) for s, o in jobs]
            for f in futs:
                f.result()
    lib_time = lib.stat().st_mtime if lib.exists() else 0.0
    if force or jobs or any(o.stat().st_mtime > lib_time for o in objs):
        tmp = lib.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
               "-lpthread", "-Xlinker", "-z,defs"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    stamp.write_text(arch + "\n")
    return lib


if __name__ == "__main__":
    print(build_native(verbose="-v" in sys.argv, force="-f" in sys.argv))
