"""Writes transport_small_fp64.npz: FP64 oracle results of the small cases.

Each case is a synthetic nebula of mocassin_gb300.nebula.small_cases() run
through the oracle at FP64 with Philox seed 2024, iteration 1.  Stored per
case: the counters, Jste summed over frequency for every cell, Jste summed
over cells for every bin, and escapedPackets summed over cells.  The GPU
FP64 path must reproduce them to 1e-12 relative.

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mocassin_gb300 import nebula  # noqa: E402
from oracle import runner  # noqa: E402

SEED = 2024
KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")


def main():
    out = {}
    for spec in nebula.small_cases():
        neb = nebula.build(spec)
        js, _, es, st = runner.run(neb, precision="fp64", seed=SEED)
        out[spec.name + "/counts"] = np.array([st[k] for k in KEYS], dtype=np.int64)
        out[spec.name + "/j_cell"] = js.sum(0)
        out[spec.name + "/j_nu"] = js.sum(1)
        out[spec.name + "/esc_nu"] = es.sum(1)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "transport_small_fp64.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
