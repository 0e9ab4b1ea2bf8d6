"""Builds libtensorly_gb300.so from csrc/*.cu with nvcc (sm_103a only).

Each translation unit is compiled in parallel to an object file under
``tensorly_gb300/_build/`` and linked into ``tensorly_gb300/libtensorly_gb300.so``.
Objects are rebuilt when their source, any header, or the flags change.
"""

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libtensorly_gb300.so")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def _nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand) and shutil.which(cand) is None:
        raise RuntimeError("nvcc not found: the GB300 library cannot be built")
    return cand


def _headers_digest():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE_DIR):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cuh", ".h")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode() + f.read())
    return h.hexdigest()


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(verbose=False, jobs=None):
    """Compile every csrc/*.cu for sm_103a and link the shared library."""
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    flags = ARCH_FLAGS + NVCC_FLAGS + ["-I" + INCLUDE_DIR, "-I" + CSRC]
    hdr = _headers_digest()
    objs, todo = [], []
    for src in _sources():
        with open(src, "rb") as f:
            key = hashlib.sha256(f.read() + hdr.encode() + " ".join(flags).encode()).hexdigest()[:16]
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + "." + key + ".o")
        objs.append(obj)
        if not os.path.exists(obj):
            todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        cmd = [nvcc] + flags + ["-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with concurrent.futures.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(compile_one, todo))
    relink = bool(todo) or not os.path.exists(LIB_PATH)
    if not relink:
        lib_m = os.path.getmtime(LIB_PATH)
        relink = any(os.path.getmtime(o) > lib_m for o in objs)
    if relink:
        cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", LIB_PATH + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    # drop stale objects from earlier flag / source versions
    keep = set(objs)
    for f in os.listdir(BUILD_DIR):
        p = os.path.join(BUILD_DIR, f)
        if p not in keep and f.endswith(".o"):
            try:
                os.remove(p)
            except OSError:
                pass
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
