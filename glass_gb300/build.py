"""Builds libglass_gb300.so from glass_gb300/csrc/*.cu with nvcc for sm_103a.

Each translation unit is compiled in parallel (one nvcc per file, a single
``-gencode``), then linked into a shared library next to this file.  The
build is incremental: an object is rebuilt when its source or any header in
csrc/ or include/ is newer.  Usage: ``python -m glass_gb300.build``.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
REPO_DIR = PACKAGE_DIR.parent
CSRC_DIR = PACKAGE_DIR / "csrc"
INCLUDE_DIR = REPO_DIR / "include"
BUILD_DIR = PACKAGE_DIR / "_build"
LIBRARY_NAME = "libglass_gb300.so"
LIBRARY_PATH = PACKAGE_DIR / LIBRARY_NAME

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-O2",
]


def find_nvcc() -> str:
    candidates = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for candidate in candidates:
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc was not found; set NVCC or put the CUDA toolkit on PATH")


def _headers_mtime() -> float:
    paths = list(CSRC_DIR.glob("*.cuh")) + list(CSRC_DIR.glob("*.h")) + list(INCLUDE_DIR.glob("*.h"))
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _compile(nvcc: str, source: Path, obj: Path, extra: list[str]) -> tuple[Path, str]:
    cmd = [nvcc, *ARCH_FLAGS, *COMMON_FLAGS, *extra, "-I", str(INCLUDE_DIR), "-c", str(source), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {source.name}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return obj, proc.stderr


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles every csrc/*.cu and links LIBRARY_PATH; returns its path."""
    nvcc = find_nvcc()
    extra = list(extra_flags or [])
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC_DIR.glob("*.cu"))
    if not sources:
        raise RuntimeError(f"no CUDA sources in {CSRC_DIR}")
    header_time = _headers_mtime()
    jobs = []
    objects = []
    for source in sources:
        obj = BUILD_DIR / (source.stem + ".o")
        objects.append(obj)
        stale = force or not obj.exists() or obj.stat().st_mtime < max(source.stat().st_mtime, header_time)
        if stale:
            jobs.append((source, obj))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as pool:
            futures = [pool.submit(_compile, nvcc, src, obj, extra) for src, obj in jobs]
            for future in futures:
                obj, log = future.result()
                if verbose and log.strip():
                    print(f"[{obj.name}] {log}", file=sys.stderr)
    link_needed = (
        force
        or bool(jobs)
        or not LIBRARY_PATH.exists()
        or LIBRARY_PATH.stat().st_mtime < max(o.stat().st_mtime for o in objects)
    )
    if link_needed:
        tmp = LIBRARY_PATH.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
        os.replace(tmp, LIBRARY_PATH)
    return LIBRARY_PATH


def main(argv: list[str] | None = None) -> int:
    args = list(sys.argv[1:] if argv is None else argv)
    force = "--force" in args
    verbose = "-v" in args or "--verbose" in args
    extra = ["-Xptxas", "-v"] if "--ptxas-info" in args else []
    path = build(force=force or bool(extra), verbose=verbose or bool(extra), extra_flags=extra)
    print(path)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
