"""Build recipe of the CUDA library: nvcc for sm_103a, in tree.

Each translation unit under ``csrc/`` is compiled in parallel to an object,
then linked into ``_lib/libtorchsim_gb300.so``. The library has a plain C
ABI (``include/torchsim_gb300.h``) and links the CUDA runtime statically, so
it needs nothing from PyTorch.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE / "csrc"
OUT = PACKAGE / "_lib"
OBJ = OUT / "obj"
LIBRARY = OUT / "libtorchsim_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(found).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build torchsim_gb300")
    return found


def sources() -> list[Path]:
    return sorted([*CSRC.glob("*.cu"), *CSRC.glob("*.cpp")])


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every CUDA/C++ source and link the shared library (incremental)."""
    OBJ.mkdir(parents=True, exist_ok=True)
    headers = [*CSRC.glob("*.h"), *CSRC.glob("*.cuh"), *(PACKAGE.parent / "include").glob("*.h")]
    compiler = nvcc()
    objects = []
    commands = []
    for src in sources():
        obj = OBJ / (src.name + ".o")
        objects.append(obj)
        if _stale(obj, [src, *headers]):
            commands.append([compiler, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        done = subprocess.run(cmd, capture_output=True, text=True)
        if done.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{done.stdout}\n{done.stderr}")
        return done

    workers = jobs or max(1, min(len(commands), os.cpu_count() or 1))
    if commands:
        with ThreadPoolExecutor(max_workers=workers) as pool:
            list(pool.map(run, commands))
    if commands or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_suffix(".so.tmp")
        run([compiler, *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart_static",
             "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(verbose=True))
