"""Build libvpmgpu.so in-tree with nvcc for sm_103a (GB300).

Each .cu translation unit compiles in parallel to an object under
flowunsteady_gb300/_build/, then one nvcc -shared link writes
flowunsteady_gb300/libvpmgpu.so.  Objects are rebuilt when their source or
any header under csrc/ or include/ is newer.
"""
from __future__ import annotations

import glob
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libvpmgpu.so")

_ELF_MACHINE = {"x86_64": 0x3E, "aarch64": 0xB7, "arm64": 0xB7}


def elf_matches_host(path: str) -> bool:
    """True when `path` is an ELF file built for this machine's architecture."""
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    want = _ELF_MACHINE.get(platform.machine())
    return want is None or int.from_bytes(head[18:20], "little") == want

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host loops over particles (validation, AoS <-> SoA staging) use OpenMP.
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-fopenmp"]
LINK_FLAGS = ["-Xcompiler", "-fopenmp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvpmgpu.so")


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_t = _headers_mtime()
    cc = nvcc()
    flags = FLAGS + list(extra_flags or [])

    def obj_of(src):
        return os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")

    def compile_one(src):
        obj = obj_of(src)
        if (not force and os.path.exists(obj) and elf_matches_host(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_t)):
            return obj, None
        cmd = [cc] + ARCH + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj, None

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(compile_one, srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if (force or not os.path.exists(LIB) or not elf_matches_host(LIB)
            or os.path.getmtime(LIB) < newest):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + LINK_FLAGS
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
