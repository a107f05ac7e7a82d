"""Writes full_size_digests.json: the oracle's digests of every output of the bench's full-size
workloads (the primitive sweep at 2^28 rows, the argsort/group-by pipeline at 2^27 rows for both
key distributions). bench.py compares its timed outputs with them after the timed region.

Run from the repository root: python tests/golden/make_full_digests.py [--sweep-n N] [--sort-n N]
(about 20 GB of host memory and a few minutes at the default sizes).
"""

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import full_size  # noqa: E402
from full_size import bench  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sweep-n", type=int, default=1 << 28)
    ap.add_argument("--sort-n", type=int, default=1 << 27)
    ap.add_argument("--out", default=os.path.join(HERE, "full_size_digests.json"))
    args = ap.parse_args()
    t0 = time.time()
    doc = {"generator": "tests/golden/make_full_digests.py (oracle/ restatement of the reference's scalar "
                        "entries; digest = bench.digest)",
           "sweep": {"n": args.sweep_n, "outputs": {}},
           "sort_groupby": {"n": args.sort_n}}
    for label, value in full_size.sweep_outputs(args.sweep_n):
        doc["sweep"]["outputs"][label] = bench.digest(value)
        print("sweep %-22s %s (%.0f s)" % (label, doc["sweep"]["outputs"][label], time.time() - t0), flush=True)
    for dist in ("uniform32", "zipf1.1"):
        outs = {}
        for label, value in full_size.sortgroup_outputs(args.sort_n, dist):
            outs[label] = bench.digest(value)
            print("%s %-26s %s (%.0f s)" % (dist, label, outs[label], time.time() - t0), flush=True)
        doc["sort_groupby"][dist] = outs
    with open(args.out, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
