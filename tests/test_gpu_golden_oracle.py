"""The four plain-method solves of the 4096^2 configuration (CG + jac_diag,
CG + jac_block, Chebyshev after 20 CG steps, PPCG with 10 inner steps) on the
GPU against the CPU oracle's committed golden runs
(tests/golden/oracle_config2_{1024,4096}.json, made by
tests/golden/make_oracle_golden.py): per-step iteration counts within +-1 and
field summaries within 1e-10 relative.

At tl_eps 1e-15 Chebyshev never meets its test on these grids: it measures the
true residual u0 - A u, whose FP64 floor lies above 1e-15 * ||r_0||, so every
step runs to tl_max_iters in the oracle (as in the reference) and must do the
same on the GPU."""
import json
import os

import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FS_RTOL = 1e-10


def _golden(n):
    path = os.path.join(HERE, "golden", f"oracle_config2_{n}.json")
    if not os.path.exists(path):
        pytest.skip(f"{path} not generated")
    return json.load(open(path))


@pytest.mark.parametrize("n", [1024, 4096])
@pytest.mark.parametrize("method", ["cg_jac_diag", "cg_jac_block", "chebyshev", "ppcg"])
def test_config2_against_oracle_golden(n, method):
    g = _golden(n)
    if method not in g["methods"]:
        pytest.skip(f"{method} not in the {n} golden file")
    m = g["methods"][method]
    deck = decks.make_deck(n=n, end_step=g["steps"], **m["deck_params"])
    recs, res = tl.run_deck(deck)
    assert res["status"] == 0, tl.last_error()
    gold = m["steps"]
    assert len(recs) == len(gold)
    for r, o in zip(recs[1:], gold[1:]):
        assert abs(r["iterations"] - o["iterations"]) <= 1, (r["step"], r["iterations"], o["iterations"])
    for k in ("vol", "mass", "ie", "temp"):
        assert recs[-1][k] == pytest.approx(gold[-1][k], rel=FS_RTOL), k
