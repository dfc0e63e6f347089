"""Golden fixtures of the CPU oracle for the configurations the reference
publishes nothing for: CG + jac_diag, CG + jac_block, Chebyshev after 20 CG
steps and PPCG with 10 inner steps on the standard deck (BASELINE config 2),
at 1024^2 for 20 timesteps and at 4096^2 for the first timestep.

The oracle is pinned against the reference's own benchmark outputs
(tests/test_oracle_golden.py); these fixtures let the GPU tests compare
against it at sizes where rerunning the oracle inside a test would take too
long.  Usage:
    python tests/golden/make_oracle_golden.py [--sizes 1024,4096] [--threads N]
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
                  "tl_preconditioner_type": "none"},
    "ppcg": {"tl_use_cg": False, "tl_use_ppcg": True, "tl_ppcg_inner_steps": 10,
             "tl_preconditioner_type": "none"},
}
STEPS = {1024: 20, 4096: 1}


def deck_for(n, method):
    return decks.make_deck(n=n, end_step=STEPS[n], **METHODS[method])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="1024,4096")
    ap.add_argument("--threads", type=int, default=None)
    args = ap.parse_args()
    for n in [int(x) for x in args.sizes.split(",")]:
        path = os.path.join(HERE, f"oracle_config2_{n}.json")
        out = {"source": "oracle/ (CPU restatement), tests/golden/make_oracle_golden.py",
               "n": n, "steps": STEPS[n], "methods": {}}
        if os.path.exists(path):
            out = json.load(open(path))
        for m in METHODS:
            if m in out["methods"]:
                continue
            steps, run = run_deck(deck_for(n, m), threads=args.threads)
            out["methods"][m] = {"deck_params": METHODS[m], "steps": steps, "wall": run["wall"],
                                 "threads": run["threads"]}
            json.dump(out, open(path, "w"), indent=1)
            print(f"{n} {m}: {[s['iterations'] for s in steps[1:]]} in {run['wall']:.1f}s", flush=True)


if __name__ == "__main__":
    main()
