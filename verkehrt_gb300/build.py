"""Builds the CUDA library libvkcuda.so in-tree, for sm_103a only.

Each translation unit under csrc/ compiles in parallel with nvcc into _build/, then links into
verkehrt_gb300/libvkcuda.so. A stamp file beside the library holds a hash of every source and
header, of this script and of the compiler flags; the library is rebuilt whenever the stamp is
missing or differs, so a library built from other sources (or copied from another machine) is
never reused. `-fmad=false` keeps every f64 multiply and add a separate IEEE operation, which
the canonical sums and the fused-equals-unfused identity rely on.
"""

import hashlib
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvkcuda.so")
STAMP = LIB + ".stamp"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include")]


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def source_hash():
    """SHA-256 over the sources, headers, this script, the flags and the host machine type."""
    h = hashlib.sha256()
    h.update(" ".join([NVCC] + ARCH + FLAGS + [platform.machine()]).encode())
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    with open(__file__, "rb") as fh:
        h.update(fh.read())
    return h.hexdigest()


def up_to_date():
    if not (os.path.exists(LIB) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as f:
        return f.read().strip() == source_hash()


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build(force=False, verbose=False):
    """Compiles and links libvkcuda.so unless its stamp matches the sources. Returns its path."""
    digest = source_hash()
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [NVCC] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        out = _run(cmd)
        if verbose and out.strip():
            sys.stderr.write(out)
        return obj

    workers = max(2, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    with open(STAMP + ".tmp", "w") as f:
        f.write(digest + "\n")
    os.replace(STAMP + ".tmp", STAMP)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
