"""Pin the CPU oracle against the reference's golden vectors
(Benchmarks/tea_bm_{1..4}.out, field_summary.f90:96-101).

The reference's published runs are plain CG, no preconditioner, tl_eps 1e-15.
Iteration counts must match exactly on every timestep; field_summary rows
within 1e-10 relative (the golden runs summed 1e6 cells naively, which alone
moves the volume by 2e-11)."""
import pytest

from tests import decks
from tests.oracle_run import run_deck

FS_RTOL = 1e-10


def _check(name):
    g = decks.golden()[name]
    steps, run = run_deck(decks.golden_deck(name))
    its = [s["iterations"] for s in steps if s["step"] > 0]
    assert its == g["iterations"]
    s0 = steps[0]
    sf = [s for s in steps if "temp" in s][-1]
    for key, gk in (("vol", "volume"), ("mass", "mass"), ("ie", "energy"), ("temp", "u")):
        assert s0[key] == pytest.approx(g["summary_step0"][gk], rel=FS_RTOL)
        assert sf[key] == pytest.approx(g["summary_final"][gk], rel=FS_RTOL)
    # the QA check of field_summary.f90:92-112 (0.001 %)
    assert abs(100.0 * sf["temp"] / g["qa_temp"] - 100.0) < 0.001
    # conduction error printed to 7 digits
    for e_or, e_g in zip([s["error_ratio"] for s in steps if s["step"] > 0], g["conduction_error"]):
        assert e_or == pytest.approx(e_g, rel=2e-6)


@pytest.mark.parametrize("name", ["tea_bm_1", "tea_bm_2", "tea_bm_3"])
def test_oracle_matches_reference_benchmarks(name):
    _check(name)


@pytest.mark.slow
def test_oracle_matches_reference_benchmark_1000():
    _check("tea_bm_4")
