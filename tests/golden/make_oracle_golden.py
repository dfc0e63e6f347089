"""Golden fixtures of the CPU oracle for the configurations the reference
publishes nothing for, on the standard deck (the 4096^2 configuration of the
scope: 20 timesteps each of CG + jac_diag, CG + jac_block, Chebyshev after
20 CG steps, and PPCG with 10 inner steps and block-Jacobi, the headline
method's preconditioner), at 1024^2 and 4096^2.

Chebyshev runs at tl_eps 1e-10 on 1024^2 and 1e-8 on 4096^2: it measures
the true residual, whose FP64 floor lies above 1e-15 * ||r_0|| on these
grids (and above 1e-10 from the third timestep on 4096^2, above 1e-9 from
the sixteenth), so at a tighter tolerance its steps run to tl_max_iters and
their iteration counts pin nothing.

Every step record carries the field summary and u at a 16 x 16 lattice of interior cells
(`u_samples`, tea_oracle --u-samples), against which the mixed-precision
solves report their per-timestep pointwise error.

The oracle is pinned against the reference's own benchmark outputs
(tests/test_oracle_golden.py); these fixtures let the GPU tests compare
against it at sizes where rerunning the oracle inside a test would take too
long (4096^2 x 20 timesteps is about an hour a method on 8 cores).  Usage:
    python tests/golden/make_oracle_golden.py [--sizes 1024,4096]
        [--methods cg_jac_diag,...] [--threads N]
Methods already present in a fixture file are kept; delete an entry to
regenerate it.
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests import decks  # noqa: E402
from tests.oracle_run import run_deck  # noqa: E402

METHODS = {
    "cg_jac_diag": {"tl_use_cg": True, "tl_preconditioner_type": "jac_diag"},
    "cg_jac_block": {"tl_use_cg": True, "tl_preconditioner_type": "jac_block"},
    "chebyshev": {"tl_use_cg": False, "tl_use_chebyshev": True, "tl_ch_cg_presteps": 20,
                  "tl_preconditioner_type": "none", "tl_eps": 1.0e-10},
    "ppcg_jac_block": {"tl_use_cg": False, "tl_use_ppcg": True, "tl_ppcg_inner_steps": 10,
                       "tl_preconditioner_type": "jac_block"},
}
STEPS = 20
U_SAMPLES = 16


# the tightest Chebyshev tolerance each grid attains on every timestep
CHEBY_EPS = {1024: 1.0e-10, 4096: 1.0e-8}


def params_for(n, method):
    p = dict(METHODS[method])
    if method == "chebyshev":
        p["tl_eps"] = CHEBY_EPS[n]
    return p


def deck_for(n, method, steps=STEPS):
    # a field summary every timestep (it only reads the fields)
    return decks.make_deck(n=n, end_step=steps, summary_frequency=1, **params_for(n, method))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="1024,4096")
    ap.add_argument("--methods", default=",".join(METHODS))
    ap.add_argument("--threads", type=int, default=None)
    args = ap.parse_args()
    for n in [int(x) for x in args.sizes.split(",")]:
        path = os.path.join(HERE, f"oracle_config2_{n}.json")
        out = {"source": "oracle/ (CPU restatement), tests/golden/make_oracle_golden.py",
               "n": n, "u_samples": U_SAMPLES, "methods": {}}
        if os.path.exists(path):
            out = json.load(open(path))
        for m in args.methods.split(","):
            if m in out["methods"]:
                continue
            steps, run = run_deck(deck_for(n, m), threads=args.threads, u_samples=U_SAMPLES)
            out["methods"][m] = {"deck_params": params_for(n, m), "end_step": STEPS, "steps": steps,
                                 "wall": run["wall"], "threads": run["threads"]}
            with open(path + ".tmp", "w") as f:
                json.dump(out, f, indent=1)
            os.replace(path + ".tmp", path)
            print(f"{n} {m}: {[s['iterations'] for s in steps[1:]]} in {run['wall']:.1f}s", flush=True)


if __name__ == "__main__":
    main()
