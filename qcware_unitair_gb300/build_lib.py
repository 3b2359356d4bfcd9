"""Build recipe for libgbsv.so (the CUDA kernels behind the C ABI).

Each ``csrc/*.cu`` translation unit is compiled for sm_103a only, in
parallel, then linked into ``_build/libgbsv.so`` beside this file.  Nothing
is installed into site-packages, so the library that Python loads is the
in-tree one.  A stamp of source hashes skips the rebuild when nothing
changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libgbsv.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build "
                       "libgbsv.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def _stamp() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH_FLAGS + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def lib_path() -> Path:
    return BUILD_DIR / LIB_NAME


def build(verbose: bool = False, force: bool = False,
          extra_flags: list[str] | None = None) -> Path:
    """Compile and link libgbsv.so; return its path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    stamp_file = BUILD_DIR / "stamp.txt"
    stamp = _stamp() + (" ".join(extra_flags) if extra_flags else "")
    out = lib_path()
    if (not force and out.exists() and stamp_file.exists()
            and stamp_file.read_text() == stamp):
        return out
    nvcc = _nvcc()
    flags = ARCH_FLAGS + NVCC_FLAGS + (extra_flags or []) + [
        f"-I{INCLUDE}", f"-I{CSRC}"]
    objs = []

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        if src.suffix == ".cpp":  # host-only code
            cmd = [_cxx(), "-O3", "-std=c++17", "-fPIC", f"-I{INCLUDE}",
                   f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compile failed on {src.name}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr, file=sys.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs),
           "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, out)
    stamp_file.write_text(stamp)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
