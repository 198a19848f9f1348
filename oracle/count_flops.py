"""Count the algorithmic FP64 operations per system-step of every workload.

Runs the operation-counting build of the CPU oracle (every +, -, *, /, sqrt
of the reference's FP64 path counts 1; ``real`` wrapper in
whfast_oracle.cpp) on a seeded sample of each workload, after a few
unmeasured steps, and writes the constants to ``roofline.json`` at the
repository root:

    python oracle/count_flops.py

The counts include the midpoint and predictor-corrector iteration counts the
sample actually takes.  bench.py measures the same constant in-run for the
roofline of its line; this file records them per workload.
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from oracle.case_json import stack  # noqa: E402
from posidonius_gb300 import ensemble as E, layout as L  # noqa: E402


def _sample(ens, k):
    idx = np.linspace(0, ens["n_sys"] - 1, k).astype(np.int64)
    out = {key: (v[idx] if isinstance(v, np.ndarray) and key != "tables" else v) for key, v in ens.items()}
    out["n_sys"] = k
    return out


def count(ens, warm, steps):
    state, _, _ = oracle.run(ens, max_steps=warm, init_physical=True, nthreads=8)
    _, done, _, cnt = oracle.run(state, max_steps=steps, flops=True)
    n = float(np.sum(done))
    return {"flops_per_system_step": cnt[0] / n, "divisions_per_system_step": cnt[1] / n,
            "sqrts_per_system_step": cnt[2] / n, "system_steps_counted": int(n)}


def main():
    from posidonius_gb300 import adjoint as A
    out = {}
    work = {
        "single (config 0: star + 3 planets, WHFast Jacobi)": (E.workload_single(), 3, 50),
        "ensemble8 (config 1: star + 7 planets)": (_sample(E.workload_ensemble8(4096), 64), 3, 20),
        "uneven (config 2: 2-10 bodies, 20% binaries)": (_sample(E.workload_uneven(16384), 256), 3, 20),
        "gradient (config 3: forward step, star + 3 planets)": (_sample(A.gradient_workload(1024)[0], 64), 3, 20),
        "large (config 4: 1024 bodies, democratic heliocentric)": (stack([E.workload_large(1021)]), 1, 1),
        "ias15 (the ensemble8 systems by IAS15)": (_sample(E.as_ias15(E.workload_ensemble8(4096), dt=0.08), 32), 5, 5),
    }
    for name, (ens, warm, steps) in work.items():
        out[name] = count(ens, warm, steps)
        print(name, out[name])
    out["_note"] = ("+ - * / sqrt each count 1 (oracle/whfast_oracle.cpp built with ORACLE_COUNT_FLOPS); "
                    "per system-step averaged over the sample after a few unmeasured steps")
    with open(os.path.join(ROOT, "roofline.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
