"""The reference's own CUDA kernels, built from its sources for sm_103a -- a GPU comparator.

TEST AND BENCHMARK INFRASTRUCTURE ONLY (like the rest of oracle/): the product package
never imports this module. bench.py uses it to time the reference's kernels on the same
GPU and workloads as this engine.

``build(reference_root)`` compiles two translation units of the reference package
gpufsm 0.1.0 (alepot55/abstraction-regret) where they lie, with nvcc, into device-code
images under ``oracle/_ref/``:

* ``src/gpufsm/backends/cuda/native/dfa.cu``             -> ``dfa_kernel`` (dfa.cu:9-29)
* ``src/gpufsm/backends/cuda/native/worklist_global.cu`` -> ``worklist_warp_kernel``
  (worklist_global.cu:289-310)

Only device code is built (``-cubin``): a cubin depends on the GPU architecture, not on
the host's, so it is built in any container that has the reference checkout and loaded
on any host with the GPU. ``Kernels`` loads an image through the CUDA driver API
(ctypes on libcuda, into the context PyTorch made current), finds a kernel by name, and
launches it with the arguments and launch shape the reference's own host functions use
(``run_dfa``, dfa.cu:32-71: 256 threads, a thread per string; ``run_worklist_warp``,
worklist_global.cu:409-468: 256 threads, a warp per string, four global bitmap buffers
of nwords words per string). Inputs are the reference's layout: int32 symbols and int32
offsets (core/packing.py:35-63).
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
NATIVE = Path("src/gpufsm/backends/cuda/native")
SOURCES = {"dfa": "dfa.cu", "worklist_global": "worklist_global.cu"}


def cubin_path(name: str) -> Path:
    return OUT / f"{name}.cubin"


def build(reference_root: str | os.PathLike = "/root/reference", force: bool = False) -> list:
    """Compile the reference's kernel sources into oracle/_ref/*.cubin (sm_103a).
    Returns the images built; nothing when the checkout is absent."""
    root = Path(reference_root)
    native = root / NATIVE
    if not native.is_dir():
        return []
    nvcc = shutil.which("nvcc") or str(Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
                                       / "bin" / "nvcc")
    import sysconfig

    includes = [str(native / "include"), sysconfig.get_paths()["include"]]
    try:
        import pybind11

        includes.append(pybind11.get_include())
    except ImportError:
        return []
    OUT.mkdir(parents=True, exist_ok=True)
    built = []
    for name, src in SOURCES.items():
        out = cubin_path(name)
        if out.exists() and not force and out.stat().st_mtime >= (native / src).stat().st_mtime:
            built.append(out)
            continue
        cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
               "-std=c++17", *[f"-I{p}" for p in includes], str(native / src), "-o", str(out)]
        subprocess.run(cmd, check=True, capture_output=True)
        built.append(out)
    return built


# ---- driver API (ctypes) -----------------------------------------------------------------

_cuda = None


def _driver():
    global _cuda
    if _cuda is None:
        lib = ctypes.CDLL("libcuda.so.1")
        v = ctypes.c_void_p
        lib.cuModuleLoad.argtypes = [ctypes.POINTER(v), ctypes.c_char_p]
        lib.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), v]
        lib.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(v), ctypes.c_uint, v]
        lib.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), v]
        lib.cuLaunchKernel.argtypes = [v, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                       ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                       ctypes.c_uint, v, ctypes.POINTER(v), v]
        lib.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        _cuda = lib
    return _cuda


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(msg.value or b'').decode()})")


class Kernels:
    """One loaded image; ``fn(name)`` is the kernel whose (mangled) name contains it."""

    def __init__(self, name: str) -> None:
        path = cubin_path(name)
        if not path.exists():
            raise FileNotFoundError(f"{path} is not built (the reference checkout was absent "
                                    f"where this copy was built)")
        lib = _driver()
        self.module = ctypes.c_void_p()
        _check(lib.cuModuleLoad(ctypes.byref(self.module), str(path).encode()), "cuModuleLoad")
        count = ctypes.c_uint()
        _check(lib.cuModuleGetFunctionCount(ctypes.byref(count), self.module),
               "cuModuleGetFunctionCount")
        fns = (ctypes.c_void_p * count.value)()
        _check(lib.cuModuleEnumerateFunctions(fns, count.value, self.module),
               "cuModuleEnumerateFunctions")
        self.functions = {}
        for f in fns:
            nm = ctypes.c_char_p()
            _check(lib.cuFuncGetName(ctypes.byref(nm), f), "cuFuncGetName")
            self.functions[(nm.value or b"").decode()] = f

    def fn(self, name: str):
        hits = [f for n, f in self.functions.items() if name in n]
        if len(hits) != 1:
            raise KeyError(f"{name}: {len(hits)} matching kernels in {list(self.functions)}")
        return hits[0]


def launch(fn, grid: int, block: int, args: list, stream: int = 0, shmem: int = 0) -> None:
    """cuLaunchKernel with ``args`` as ctypes values (c_void_p device pointers, c_int)."""
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
                                              for a in args])
    _check(_driver().cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, shmem, ctypes.c_void_p(stream),
                                    params, None), "cuLaunchKernel")


def dfa_kernel_args(trans, accept, data, offsets, n, num_states, start, flags, lens):
    """Arguments of dfa_kernel (dfa.cu:9-12), device pointers as integers."""
    p = ctypes.c_void_p
    return [p(trans), p(accept), p(data), p(offsets), ctypes.c_int(n), ctypes.c_int(num_states),
            ctypes.c_int(start), p(flags), p(lens)]


def worklist_warp_args(srp, stg, ssy, erp, etg, acc_words, data, offsets, n, start, uses_any,
                       nwords, cur, nxt, frontier, newb, flags, lens):
    """Arguments of worklist_warp_kernel (worklist_global.cu:289-296)."""
    p = ctypes.c_void_p
    return [p(srp), p(stg), p(ssy), p(erp), p(etg), p(acc_words), p(data), p(offsets),
            ctypes.c_int(n), ctypes.c_int(start), ctypes.c_int(uses_any), ctypes.c_int(nwords),
            p(cur), p(nxt), p(frontier), p(newb), p(flags), p(lens)]


if __name__ == "__main__":
    print([str(p) for p in build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference",
                                 force=True)])
