"""Builds the CPU oracle liboracle.so (test infrastructure: the checker and the CPU baseline).

-O3 -ffp-contract=off: no multiply-add contraction, as the reference's scalar entries compute
(every f64 product is rounded before it is added). A stamp file beside the library holds a hash
of the sources, this script and the host machine type; a missing or different stamp rebuilds.
"""

import hashlib
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
STAMP = LIB + ".stamp"
SRCS = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "elementwise.c"), os.path.join(HERE, "families.c")]
HDR = os.path.join(HERE, "oracle.h")
CFLAGS = ["-O3", "-ffp-contract=off", "-std=c11", "-fPIC", "-shared"]


def source_hash():
    h = hashlib.sha256()
    h.update(" ".join(CFLAGS + [os.environ.get("CC", "gcc"), platform.machine()]).encode())
    for p in SRCS + [HDR, __file__]:
        with open(p, "rb") as f:
            h.update(os.path.basename(p).encode())
            h.update(f.read())
    return h.hexdigest()


def build(force=False):
    digest = source_hash()
    if not force and os.path.exists(LIB) and os.path.exists(STAMP):
        with open(STAMP) as f:
            if f.read().strip() == digest:
                return LIB
    cc = os.environ.get("CC", "gcc")
    tmp = LIB + ".tmp"
    cmd = [cc] + CFLAGS + ["-o", tmp] + SRCS + ["-lm"]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + p.stdout)
    os.replace(tmp, LIB)
    with open(STAMP + ".tmp", "w") as f:
        f.write(digest + "\n")
    os.replace(STAMP + ".tmp", STAMP)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
