"""Regenerate tests/golden/iteration_counts.json from the reference's results.

The reference ships no unit tests; its only data that pin numerical results
are the benchmark timings in ``results/scaling_data*.npz`` (written by
scaling_jax.py:151-156).  For each grid size N they hold the total time of
``time_integration`` to t_final=0.2 and that time divided by the number of
iterations (scaling_jax.py:70), so ``round(total / per_iteration)`` is the
reference's iteration count for ``setup_ics(N, N//16)``, gamma=5/3,
handle_boundaries=True (scaling_jax.py:86-93, 236).

Usage: python tests/golden/make_golden.py <path of the reference checkout>
"""
import json
import os
import sys

import numpy as np


def main(ref_root):
    out = {"source": "results/scaling_data.npz (execution_times / execution_times_per_iteration)",
           "t_final": 0.2, "gamma": 5.0 / 3.0, "num_injection_cells": "N // 16",
           "handle_boundaries": True, "counts": {}, "cross_check": {}}
    d = np.load(os.path.join(ref_root, "results", "scaling_data.npz"))
    for n, tot, per in zip(d["num_cells_list"], d["execution_times"],
                           d["execution_times_per_iteration"]):
        ratio = float(tot) / float(per)
        assert abs(ratio - round(ratio)) < 1e-3, (n, ratio)
        out["counts"][str(int(n))] = int(round(ratio))
    # the GSPMD run (same step, 2x2 sharded) must give the same counts
    for name in ("scaling_data_sharding.npz",):
        d2 = np.load(os.path.join(ref_root, "results", name))
        out["cross_check"][name] = {
            str(int(n)): int(round(float(t) / float(p)))
            for n, t, p in zip(d2["num_cells_list"], d2["execution_times"],
                               d2["execution_times_per_iteration"])}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "iteration_counts.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(json.dumps(out["counts"]), json.dumps(out["cross_check"]))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
