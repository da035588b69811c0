"""Build recipe for libpermgpu.so (sm_103a) — no cmake, parallel nvcc.

Each ``csrc/*.cu`` translation unit is compiled to an object under
``csrc/_build/`` with ``-gencode arch=compute_103a,code=sm_103a`` and the
objects are linked into ``permgpu/libpermgpu.so``.  Objects are rebuilt only
when their source or any header in ``csrc/`` / ``include/`` is newer.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent                     # rivin-perm_gb300/
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD = CSRC / "_build"
LIB = PKG_DIR / "libpermgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found (CUDA toolkit required to build libpermgpu)")


def _newest_header() -> float:
    stamps = [p.stat().st_mtime for p in CSRC.glob("*.h")]
    stamps += [p.stat().st_mtime for p in CSRC.glob("*.cuh")]
    stamps += [p.stat().st_mtime for p in INCLUDE.glob("*.h")]
    return max(stamps) if stamps else 0.0


def build(verbose: bool = False, jobs: int | None = None,
          extra_flags: list[str] | None = None, lib_path: Path | None = None,
          build_dir: Path | None = None) -> Path:
    """Compile every CUDA translation unit and link libpermgpu.so.

    ``extra_flags`` (e.g. tuning macros), ``lib_path`` and ``build_dir``
    allow building variants of the library side by side."""
    nvcc = _nvcc()
    LIB = Path(lib_path) if lib_path else globals()["LIB"]
    BUILD = Path(build_dir) if build_dir else globals()["BUILD"]
    BUILD.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    hdr = _newest_header()
    flags = ARCH + NVCC_FLAGS + list(extra_flags or [])
    # nvcc's intermediate files go to a folder of the build tree
    tmp = BUILD / "tmp"
    tmp.mkdir(parents=True, exist_ok=True)
    env = dict(os.environ, TMPDIR=str(tmp))

    def compile_one(src: Path):
        obj = BUILD / (src.stem + ".o")
        if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr):
            return obj, False, ""
        cmd = [nvcc, *flags, "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True, env=env)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")
        return obj, True, res.stderr

    jobs = jobs or max(1, min(len(sources), os.cpu_count() or 1))
    objs, rebuilt = [], False
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, did, log in ex.map(compile_one, sources):
            objs.append(obj)
            rebuilt |= did
            if verbose and did:
                print(f"[permgpu] compiled {obj.name}")
                if log.strip():
                    print(log)
    if rebuilt or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True, env=env)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
        os.replace(tmp, LIB)
        if verbose:
            print(f"[permgpu] linked {LIB}")
    return LIB


if __name__ == "__main__":
    import sys
    build(verbose="-v" in sys.argv)
