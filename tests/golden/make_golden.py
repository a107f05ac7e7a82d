#!/usr/bin/env python3
"""Writes the golden fixtures of this directory.

known_answers.json  known answers that antiguru/verkehrt's own tests and README hold for the
                    kernel-table primitives, transcribed with the file:line they come from (the
                    reference is Rust and cannot be built or imported here, so these are read as
                    text; the oracle reproduces every one of them, see test_oracle_golden.py).
oracle_vectors.npz  outputs of the C oracle on small seeded inputs (the reference's generators),
                    so that GPU tests compare against committed values and a change of the
                    oracle shows up as a failing CPU test.

Run from the repository root: python tests/golden/make_golden.py
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

KNOWN = {
    "splitmix64(0)": {"value": "0xe220a8397b1dcdaf", "source": "src/kernels/tests.rs:1167-1181"},
    "rand_i64(2, 0)": {"value": [-2152535657050944081, -7995527694508729151],
                       "source": "tests/programs/random.dd:4-9"},
    "canonical sum of the 35-row mixed-magnitude vector": {
        "value": "0x4049147ae147ae14", "source": "src/kernels/tests.rs:761-791"},
    "README example": {
        "program": "x = rand_f64(1000000, 1); y = rand_f64(1000000, 2); sum(x*y); count(x > 0.5); "
                   "length(filter(x, |v| v > 0.99))",
        "value": {"dot": 249724.39002046228, "count_gt_0.5": 499521, "filter_gt_0.99_length": 9851},
        "source": "README.md:64-69"},
    "arrays.dd dot": {"value": 32.0, "source": "tests/programs/arrays.dd"},
    "grouping.dd group_id": {"input": [7, -1, 7, 3, -1, 7], "value": [0, 1, 0, 2, 1, 0],
                             "source": "tests/programs/grouping.dd"},
    "argsort i64 extremes": {"input": [2**63 - 1, 0, -2**63, -1, 2**63 - 1, -2**63, 0, -1],
                             "value": [2, 5, 3, 7, 1, 6, 0, 4],
                             "source": "src/kernels/scalar/index/tests.rs:246-266"},
}


def bits(x):
    return np.float64(x).view(np.uint64)


def vectors():
    n = 3001
    x, y = oracle.rand_f64(n, 1), oracle.rand_f64(n, 2)
    v = (oracle.rand_i64(n, 5) & ((1 << 21) - 1)) - (1 << 20)
    starts = (oracle.rand_i64(n, 6).view(np.uint64) % np.uint64(7)) == 0
    src = oracle.rand_i64(4096, 3)
    idx = (oracle.rand_i64(n, 4) & 4095).astype(np.int64)
    keys = (oracle.rand_i64(n, 9).view(np.uint64) % np.uint64(1000)).astype(np.int64) - 500
    gkeys = (oracle.rand_i64(n, 10).view(np.uint64) % np.uint64(50)).astype(np.int64)
    ids = oracle.group_id_i64(gkeys)
    nb = int(oracle.reduce_max_i64(ids)) + 1
    mask = oracle.rand_i64(n, 12) % 3 == 0
    out = {
        "x": x, "y": y, "v": v, "starts": starts, "src": src, "idx": idx, "keys": keys,
        "gkeys": gkeys, "mask": mask,
        "reduce_add_bits": bits(oracle.reduce_add_f64(x)),
        "dot_bits": bits(oracle.dot_f64(x, y)),
        "sumsq_bits": bits(oracle.sumsq_f64(x)),
        "count_gt_0.5": np.int64(oracle.count_cmp_f64(x, "gt", 0.5)),
        "filter_gt_0.9": oracle.filter_cmp_f64(x, "gt", 0.9),
        "min_bits": bits(oracle.reduce_min_f64(x)), "max_bits": bits(oracle.reduce_max_f64(x)),
        "argmin": np.int64(oracle.argmin_f64(x)), "argmax": np.int64(oracle.argmax_f64(x)),
        "scan_add": oracle.scan_add_i64(v), "scan_by_add": oracle.scan_by_add_i64(v, starts),
        "prev": oracle.prev_i64(v, 7), "gather": oracle.gather(src, idx),
        "argsort": oracle.argsort_i64(keys), "group_id": ids,
        "histogram": oracle.histogram(ids, nb), "reduce_into": oracle.reduce_into_add_i64(ids, v, nb),
        "compress": oracle.compress(x, mask), "where": oracle.where(mask),
    }
    return out


def main():
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(KNOWN, f, indent=1)
        f.write("\n")
    np.savez_compressed(os.path.join(HERE, "oracle_vectors.npz"), **vectors())


if __name__ == "__main__":
    main()
