"""The mixed-precision form (FP32 inner CG, FP64 iterative refinement) against
the plain FP64 GPU solve and the CPU oracle.

Bar: the same field_summary as plain FP64 CG within 1e-10 relative, and the
same final FP64 residual test (||u0 - A u|| below tl_eps * ||r_0||, or the FP64
floor).  The per-timestep error of u against the FP64 solution is checked and
reported."""
import numpy as np
import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks
from tests.oracle_run import run_deck as oracle_run

pytestmark = pytest.mark.gpu

FS_RTOL = 1e-10


def _solve_steps(deck, steps):
    cfg = tl.parse_deck(deck)
    out = []
    with tl.Chunk(cfg) as ch:
        ch.start()
        for _ in range(steps):
            info = ch.timestep()
            out.append((info, ch.field_summary(), ch.interior("u").copy()))
    return out


@pytest.mark.parametrize("precond", ["none", "jac_diag"])
@pytest.mark.parametrize("shape", [(64, 48), (200, 150)])
def test_mixed_matches_fp64(precond, shape):
    base = dict(x_cells=shape[0], y_cells=shape[1], end_step=3, tl_preconditioner_type=precond)
    fp64 = _solve_steps(decks.make_deck(**base), 3)
    mixed = _solve_steps(decks.make_deck(tl_precision="mixed", **base), 3)
    for step, ((i64, s64, u64), (imx, smx, umx)) in enumerate(zip(fp64, mixed), start=1):
        assert imx["status"] == 0
        assert imx["outer_iters"] >= 1 and imx["inner_iters"] >= 1
        for a, b in zip(s64, smx):
            assert b == pytest.approx(a, rel=FS_RTOL), step
        err = np.max(np.abs(umx - u64)) / np.max(np.abs(u64))
        print(f"step {step}: outer {imx['outer_iters']} inner {imx['inner_iters']} "
              f"(fp64 {i64['iterations']}) max|du|/max|u| = {err:.2e}")
        assert err < 1e-9


def test_mixed_matches_oracle_field_summary():
    deck = decks.make_deck(x_cells=96, y_cells=96, end_step=4, tl_preconditioner_type="jac_diag")
    steps, _ = oracle_run(deck)
    recs, res = tl.run_deck(deck.replace("*endtea", "tl_precision mixed\n*endtea"))
    assert res["status"] == 0
    for k in ("vol", "mass", "ie", "temp"):
        assert recs[-1][k] == pytest.approx(steps[-1][k], rel=FS_RTOL)


def test_mixed_reaches_tl_eps_on_the_true_residual():
    deck = decks.make_deck(x_cells=128, y_cells=128, end_step=1, tl_preconditioner_type="jac_diag",
                           tl_eps=1e-12, tl_precision="mixed")
    (info, _, _), = _solve_steps(deck, 1)
    assert info["error_ratio"] < 1e-12


@pytest.mark.parametrize("precond,shape", [("none", (96, 80)), ("jac_diag", (96, 80)), ("jac_block", (96, 80)),
                                            ("jac_block", (97, 43)), ("jac_diag", (131, 58))])
def test_mixed_ppcg_matches_fp64(precond, shape):
    """PPCG with its polynomial preconditioner (the 10 inner steps) in FP32:
    the outer flexible CG stays FP64 and reaches the same answer (odd sizes:
    ragged float4 lanes and a partial last block-Jacobi strip)."""
    base = dict(x_cells=shape[0], y_cells=shape[1], end_step=3, tl_preconditioner_type=precond, tl_use_cg=False,
                tl_use_ppcg=True, tl_ppcg_inner_steps=10, tl_ch_cg_presteps=10, tl_ch_cg_epslim=1.0e10)
    fp64 = _solve_steps(decks.make_deck(**base), 3)
    mixed = _solve_steps(decks.make_deck(tl_precision="mixed", **base), 3)
    for step, ((i64, s64, u64), (imx, smx, umx)) in enumerate(zip(fp64, mixed), start=1):
        assert imx["status"] == 0
        for a, b in zip(s64, smx):
            assert b == pytest.approx(a, rel=FS_RTOL), step
        err = np.max(np.abs(umx - u64)) / np.max(np.abs(u64))
        print(f"ppcg {precond} step {step}: outer its fp64 {i64['iterations']} mixed {imx['iterations']}, "
              f"max|du|/max|u| = {err:.2e}, eigenvalues fp64 {i64['eigmin']:.6g} {i64['eigmax']:.6g} "
              f"mixed {imx['eigmin']:.6g} {imx['eigmax']:.6g}")
        assert err < 1e-9
        # the first solve's CG presteps run in FP32 there: the same switch
        # step and the same spectrum estimate from their Lanczos coefficients
        assert imx["switch_n"] == i64["switch_n"]
        assert imx["eigmin"] == pytest.approx(i64["eigmin"], rel=1e-3)
        assert imx["eigmax"] == pytest.approx(i64["eigmax"], rel=1e-3)


def _fusion_runs(precond, settings):
    deck = decks.make_deck(x_cells=600, y_cells=150, end_step=2, tl_preconditioner_type=precond, tl_use_cg=False,
                           tl_use_ppcg=True, tl_ppcg_inner_steps=10, tl_ch_cg_presteps=10,
                           tl_ch_cg_epslim=1.0e10, tl_precision="mixed")
    runs = {}
    for key in settings:
        cfg = tl.parse_deck(deck)
        with tl.Chunk(cfg) as ch:
            ch.set_inner_fusion(*key)
            ch.start()
            infos = [ch.timestep() for _ in range(2)]
            its = [i["iterations"] for i in infos]
            runs[key] = (its, ch.interior("u").copy(), ch.field_summary(), [i["ppcg_inner_iters"] for i in infos])
    return runs


@pytest.mark.parametrize("precond", ["none", "jac_diag", "jac_block"])
def test_fused_inner_steps_are_bitwise_equal(precond):
    """The temporally blocked inner steps (2-5 per pass, any share size)
    give the bits of one kernel per inner step; 600 x 150 cells make several
    column bands, a partial last strip and many shares.  (The outer
    rrn sum stays in its own kernel here: fold_rrn off.)"""
    runs = _fusion_runs(precond, [(1, 32, False), (2, 32, False), (3, 4, False), (4, 4, False),
                                  (4, 1, False), (2, 7, False), (4, 0, False), (5, 0, False), (5, 3, False)])
    its0, u0, fs0, inner0 = runs[(1, 32, False)]
    for key, (its, u, fs, inner) in runs.items():
        assert its == its0, key
        assert inner == inner0, key
        assert np.array_equal(u, u0), key
        assert fs == fs0, key


@pytest.mark.parametrize("precond", ["jac_diag", "jac_block"])
def test_folded_rrn_matches_to_round_off(precond):
    """With the outer (r - r_store).z summed inside the last fused pass the
    sum runs in another order: the solve must agree to round-off."""
    runs = _fusion_runs(precond, [(1, 32, False), (4, 0, True), (3, 5, True), (2, 1, True)])
    its0, u0, fs0, inner0 = runs[(1, 32, False)]
    for key, (its, u, fs, inner) in runs.items():
        assert all(abs(a - b) <= 1 for a, b in zip(its, its0)), key
        # the folded pass counts the outer iterations as the rrn pass does
        assert all(abs(a - b) <= 10 for a, b in zip(inner, inner0)), key
        assert np.max(np.abs(u - u0)) / np.max(np.abs(u0)) < 1e-12, key
        for a, b in zip(fs, fs0):
            assert a == pytest.approx(b, rel=1e-12), key


def test_inner_fusion_rejects_bad_settings():
    cfg = tl.parse_deck(decks.make_deck(x_cells=32, y_cells=32, end_step=1))
    with tl.Chunk(cfg) as ch:
        for bad in [(0, 32, 1), (6, 32, 1), (2, -1, 1)]:
            with pytest.raises(tl.TeaLeafError):
                ch.set_inner_fusion(*bad)
