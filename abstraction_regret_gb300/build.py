"""Build ``libgbfsm.so`` (the CUDA kernels and the C ABI) for sm_103a with nvcc.

Each translation unit under ``csrc/`` is compiled in parallel into ``_build/`` and
linked into ``abstraction_regret_gb300/libgbfsm.so`` (static CUDA runtime, so the library
only needs the driver). Host code uses no architecture-specific flags, so the same
recipe builds on x86_64 and aarch64.

    python -m abstraction_regret_gb300.build [--force]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "_build"
LIB = PKG / "libgbfsm.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--use_fast_math"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbfsm")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sources() + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + sorted(
        INCLUDE.glob("*.h")
    )


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _compile(src: Path, extra: list[str], obj_dir: Path = OUT_DIR) -> Path:
    obj = obj_dir / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stderr}\n{res.stdout}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None,
          out: Path | None = None) -> Path:
    """Compile every ``csrc/*.cu`` and link ``libgbfsm.so``; returns its path.

    ``extra`` adds nvcc flags (e.g. ``-DGBFSM_PERSIST_MIN_BLOCKS=4`` to build a tuning
    variant); ``out`` writes the library somewhere else than the package directory (load
    it with ``GBFSM_LIBRARY=<path>``).
    """
    lib = Path(out) if out else LIB
    if not force and out is None and not extra and up_to_date():
        return LIB
    obj_dir = OUT_DIR if out is None else lib.parent / (lib.stem + "_objs")
    obj_dir.mkdir(parents=True, exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as pool:
        objs = list(pool.map(lambda s: _compile(s, extra, obj_dir), srcs))
    tmp = lib.with_suffix(f".so.{os.getpid()}.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link of libgbfsm.so failed:\n{res.stderr}\n{res.stdout}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--force", action="store_true", help="rebuild even if up to date")
    ap.add_argument("--ptxas-info", action="store_true",
                    help="print registers / spills / shared memory per kernel (-Xptxas -v)")
    ap.add_argument("--define", "-D", action="append", default=[],
                    help="preprocessor define for a tuning variant, e.g. GBFSM_PERSIST_MIN_BLOCKS=4")
    ap.add_argument("--out", default=None, help="write the library to this path instead")
    args = ap.parse_args(argv)
    defines = [f"-D{d}" for d in args.define]
    extra = ["-Xptxas", "-v"] if args.ptxas_info else []
    if args.ptxas_info:
        OUT_DIR.mkdir(parents=True, exist_ok=True)
        for src in sources():
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-c", str(src), "-o",
                   str(OUT_DIR / (src.stem + ".o"))]
            res = subprocess.run(cmd, capture_output=True, text=True)
            sys.stdout.write(res.stderr)
            if res.returncode:
                return res.returncode
    build(force=args.force, verbose=True, extra=defines or None,
          out=Path(args.out) if args.out else None)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
