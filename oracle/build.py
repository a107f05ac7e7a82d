"""Builds the CPU oracle liboracle.so (test infrastructure: the checker and the CPU baseline).

-O3 -ffp-contract=off: no multiply-add contraction, as the reference's scalar entries compute
(every f64 product is rounded before it is added).
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRCS = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "elementwise.c")]
HDR = os.path.join(HERE, "oracle.h")


def build(force=False):
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(max(os.path.getmtime(f) for f in SRCS), os.path.getmtime(HDR),
                                            os.path.getmtime(__file__))):
        return LIB
    cc = os.environ.get("CC", "gcc")
    tmp = LIB + ".tmp"
    cmd = [cc, "-O3", "-ffp-contract=off", "-std=c11", "-fPIC", "-shared", "-o", tmp] + SRCS + ["-lm"]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + p.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
