"""Measures the iterations aphros's CG (SolverConjugate, linear.ipp:24-129,
restated by the oracle) needs to reach ||r||/||b|| = 1e-10 from a zero guess
on the 64-bubble field (radii 0.02-0.05, density ratio 1000, Taylor-Green +
noise) at 64^3, 128^3 and 256^3, and fits iters = a * n^b.  The benchmark's
CPU baseline extrapolates the 512^3 solve with this fit.  Test
infrastructure: run on the host, writes oracle/data/cg_iterations.json.

    python oracle/data/make_cg_iterations.py [--sizes 64 128 256]
"""
import argparse
import json
import math
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from aphros_gb300 import workload  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cg_iterations.json")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", type=int, nargs="*", default=[64, 128, 256])
    args = ap.parse_args()
    rows = []
    for n in args.sizes:
        case = workload.config("c3", n=n)
        e, _, _ = oracle.assemble_projection(n, case.h, case.dt, case.alpha, case.rho1,
                                             case.rho2, case.flux)
        t0 = time.time()
        _, info = oracle.cg_solve(n, case.h, e, oracle.rel_tol(e, case.h, 1e-10),
                                  nthreads=os.cpu_count() or 1)
        rows.append({"n": n, "iters": int(info.iter), "seconds": time.time() - t0})
        print(rows[-1], flush=True)
    ln = np.log([r["n"] for r in rows])
    li = np.log([r["iters"] for r in rows])
    b, la = np.polyfit(ln, li, 1)
    out = {"workload": "c3 bubble field (64 spheres, r 0.02-0.05, ratio 1000), "
                       "||r||/||b|| = 1e-10, zero guess, oracle CG",
           "rows": rows, "fit": {"a": math.exp(la), "b": b},
           "iters_512": int(round(math.exp(la) * 512 ** b))}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
