"""Build recipe for the native library ``libclode_gb300.so`` (in-tree, no cmake).

Steps:
  1. embed the NVRTC device headers (``csrc/device``) into
     ``_build/device_headers.inc`` so the library carries its kernel sources;
  2. compile the host translation units and the ahead-of-time kernels with
     nvcc for sm_103a, in parallel;
  3. link a shared library against the static CUDA runtime and libdl (NVRTC is
     opened at run time), so the library loads on hosts without a driver.

``python -m clode_gb300.build`` builds; ``build(force=True)`` rebuilds.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
DEVICE_DIR = os.path.join(CSRC, "device")
HOST_DIR = os.path.join(CSRC, "host")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libclode_gb300.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the native library cannot be built")


def _cuda_root(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def device_header_files() -> list[str]:
    return sorted(fn for fn in os.listdir(DEVICE_DIR) if fn.endswith((".cuh", ".h")))


def _write_device_headers() -> str:
    out = os.path.join(BUILD_DIR, "device_headers.inc")
    names = device_header_files()
    lines = ["// generated by clode_gb300/build.py from csrc/device; do not edit", ""]
    lines.append(f"static const int kDeviceHeaderCount = {len(names)};")
    lines.append("static const char *const kDeviceHeaderNames[] = {" + ", ".join(f'"{n}"' for n in names) + "};")
    lines.append("static const char *const kDeviceHeaderSources[] = {")
    for n in names:
        with open(os.path.join(DEVICE_DIR, n)) as f:
            text = f.read()
        # split into chunks: some compilers cap the length of one string literal
        chunks = [text[i:i + 12000] for i in range(0, len(text), 12000)] or [""]
        lines.append("    " + " ".join(f'R"CLODE_SRC({c})CLODE_SRC"' for c in chunks) + ",")
    lines.append("};")
    content = "\n".join(lines) + "\n"
    if not os.path.exists(out) or open(out).read() != content:
        with open(out, "w") as f:
            f.write(content)
    return out


def _sources() -> list[str]:
    return [os.path.join(HOST_DIR, fn) for fn in ("runtime.cpp", "simulator.cpp", "aot_kernels.cu", "order.cu", "noalloc.cu",
                                                  "mlp.cu", "mlp_net.cpp")]


def _fingerprint(flags: list[str]) -> str:
    h = hashlib.sha256(" ".join(flags).encode())
    files = _sources() + [os.path.join(HOST_DIR, "common.hpp"), os.path.join(HOST_DIR, "mlp.hpp"),
                          os.path.join(HERE, "..", "include", "clode_gb300.h")]
    files += [os.path.join(DEVICE_DIR, n) for n in device_header_files()]
    for fn in files:
        with open(fn, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def library_path() -> str:
    return os.path.join(BUILD_DIR, LIB_NAME)


def build(force: bool = False, verbose: bool = False) -> str:
    """Build the native library if any source changed; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    root = _cuda_root(nvcc)
    _write_device_headers()
    common = ["-std=c++17", "-O2", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              f"-I{BUILD_DIR}", f"-I{os.path.join(root, 'include')}"] + ARCH_FLAGS
    lib = library_path()
    stamp = lib + ".stamp"
    fp = _fingerprint(common)
    if not force and os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read() == fp:
        return lib

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        cmd = [nvcc] + common + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=6) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [nvcc, "-shared", "-cudart", "static"] + ARCH_FLAGS + objs + ["-o", tmp, "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    with open(stamp, "w") as f:
        f.write(fp)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
