"""Autotuner for the Householder reduction's variant and the mixed path's
back-transformation kernel.

For every matrix-size class of the uneven workloads (cubic2d L = 12..32,
triangular L = 12..24: n = 144, 256, 324, 400, 576, 1024) and both
precisions, times every compiled reduction variant (fkg_set_tuning: the
one-stage panel widths and, for the mixed path, the two-stage reduction) on a
batch of random configurations with CUDA events around the launches
(fkg_profile / fkg_stage_time), keeps the fastest and writes the table as
JSON. A variant's time is the sum of all stages of the solve (reduction,
tridiagonal eigenproblem, back-transformation, refinement): the two-stage
reduction moves work into the back-transformation (the band stage's
reflectors). For the mixed path it then times the two back-transformation
kernels (mma.sync with the block of Z in shared memory, tcgen05 with
tensor-memory accumulators; fkg_set_tuning_back) per size class under the
chosen reduction. `Solver(..., tuning=path)` (default: the table shipped next
to this file, when present) applies it with fkg_set_tuning.

Run on the GPU:  python -m fk_mc_gb300.autotune --out fk_mc_gb300/tuning_gb300.json
"""
import argparse
import json
import os

import numpy as np

DEFAULT_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json")
CLASSES = [("cubic2d", 12), ("cubic2d", 16), ("triangular", 18), ("cubic2d", 20), ("cubic2d", 24), ("cubic2d", 32)]
VARIANTS = {"mixed": [4, 8, 16, "two-stage"], "f64": [2, 4]}  # panel widths (or two-stage), index = variant
STAGES = ("reduce", "trieig", "back", "refine")
BACK_VARIANTS = {0: "mma.sync", 1: "tcgen05"}       # back-transformation kernels of the mixed path


def tune(batch=None, reps=3, seed=1):
    from .solver import Solver
    table = {"device": None, "entries": []}
    import torch
    table["device"] = torch.cuda.get_device_name(0)
    if batch is None:  # two chains per SM: the occupancy the kernels are used at
        batch = 2 * torch.cuda.get_device_properties(0).multi_processor_count
    rng = np.random.default_rng(seed)
    for prec, widths in VARIANTS.items():
        s = Solver(max_n=1024, max_batch=batch, precision=prec, tuning=None)
        s.set_graphs(False)
        for kind, L in CLASSES:
            n = s.set_lattice(0, kind, L)
            f = rng.integers(0, 2, (batch, n))
            diag = (-1.0 + 2.0 * f).ravel()
            ids = np.zeros(batch, np.int32)
            times = []
            for v in range(len(widths)):
                s.set_tuning(prec, n, v)
                s.eigh_logz(ids, diag, 4.0)  # warm
                s.profile(True)
                for _ in range(reps):
                    s.eigh_logz(ids, diag, 4.0)
                times.append(sum(s.stage_time(st)[0] for st in STAGES) / reps)
                s.profile(False)
            best = int(np.argmin(times))
            table["entries"].append({"precision": prec, "n_max": n, "variant": best, "panel_width": widths[best],
                                     "ms_per_solve": [round(t, 4) for t in times], "batch": batch})
            if prec == "mixed":
                s.set_tuning(prec, n, best)
                bt = []
                for v in sorted(BACK_VARIANTS):
                    s.set_tuning_back(n, v)
                    s.eigh_logz(ids, diag, 4.0)  # warm
                    s.profile(True)
                    for _ in range(reps):
                        s.eigh_logz(ids, diag, 4.0)
                    bt.append(s.stage_time("back")[0] / reps)
                    s.profile(False)
                best = int(np.argmin(bt))
                table["entries"].append({"stage": "back", "n_max": n, "variant": best,
                                         "kernel": BACK_VARIANTS[best], "ms_per_solve": [round(t, 4) for t in bt],
                                         "batch": batch})
                s.set_tuning_back(n, -1)
            s.set_tuning(prec, n, -1)
        s.close()
    return table


def apply(solver, path=DEFAULT_TABLE):
    """Apply a tuning table to a Solver (entries for its own sizes; others keep the default)."""
    if not path or not os.path.exists(path):
        return False
    table = json.load(open(path))
    for e in table.get("entries", []):
        if e.get("stage") == "back":
            solver.set_tuning_back(e["n_max"], e["variant"])
        else:
            solver.set_tuning(e["precision"], e["n_max"], e["variant"])
    return True


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_TABLE)
    ap.add_argument("--batch", type=int, default=None)
    args = ap.parse_args()
    t = tune(batch=args.batch)
    with open(args.out, "w") as fh:
        json.dump(t, fh, indent=1)
    print(json.dumps(t))
