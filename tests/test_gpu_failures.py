"""Failure paths of the solve, each caused on the host and none by a GPU fault.

The reference aborts the run on an eigenvalue failure (tea_solve.f90:185)
and on any CUDA error (cuda_errors.cu:163-182); here the tl_* calls return a
status instead and leave the context usable:
  * a warm-start model of NaNs: the network's direction is dropped and the
    solve starts from the increment history (or from u = u^n on the first
    step), with the same answer as without the network;
  * tl_max_iters reached: TL_WARN_MAXITER with the iterations done (for
    mixed CG: an FP32 inner solve reached it);
  * a NaN in the deck's data (one cell of energy set from the host): the
    Krylov scalars turn NaN and the solve stops with TL_ERR_BREAKDOWN at its
    first exit test instead of carrying the NaN to tl_max_iters;
  * a device allocation that fails (simulated by tl_test_fail_alloc, which
    makes the nth allocation report cudaErrorMemoryAllocation): TL_ERR_ALLOC,
    nothing allocated before it is kept, and the next attempt succeeds.
After each failure a fresh solve on the same process gives the plain answer."""
import ctypes as C

import numpy as np
import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks

pytestmark = pytest.mark.gpu

SUMMARY = ("vol", "mass", "ie", "temp")
MIB = 1 << 20


def _chunk(deck):
    ch = tl.Chunk(tl.parse_deck(deck))
    ch.start()
    return ch


def _steps(ch, k, dt=0.004):
    out = []
    for _ in range(k):
        ch.set_dt(dt)
        info = ch.timestep()
        out.append((info, ch.field_summary()))
    return out


def test_nan_model_falls_back_to_history_start():
    lib = tl.load()
    deck = decks.make_deck(x_cells=96, y_cells=80, end_step=4, tl_preconditioner_type="jac_diag")
    prev = _chunk(deck.replace("*endtea", "tl_warm_start prev\n*endtea"))
    ref = _steps(prev, 4)
    prev.close()
    ch = _chunk(deck.replace("*endtea", "tl_warm_start learned\n*endtea"))
    nan = np.full(lib.tl_warm_start_param_count(), np.nan, dtype=np.float32)
    assert lib.tl_set_warm_start_model(ch._h, C.c_void_p(nan.ctypes.data), nan.size) == 0, tl.last_error()
    got = _steps(ch, 4)
    ch.close()
    assert got[0][0]["warm_used"] == 0  # no history yet: u = u^n
    for (gi, gs), (ri, rs) in zip(got, ref):
        assert gi["status"] == tl.TL_OK
        assert gi["iterations"] == ri["iterations"]
        assert gi["warm_used"] == ri["warm_used"]
        assert gs == rs  # the same start, so the same bits


@pytest.mark.parametrize("method", [
    {"tl_use_cg": True, "tl_preconditioner_type": "jac_diag"},
    {"tl_use_cg": False, "tl_use_ppcg": True, "tl_ppcg_inner_steps": 10,
     "tl_preconditioner_type": "jac_block", "tl_ch_cg_presteps": 10, "tl_ch_cg_epslim": 1e10},
    {"tl_use_cg": True, "tl_preconditioner_type": "jac_diag", "tl_precision": "mixed"},
])
def test_max_iters_reports_a_warning(method):
    m = dict(method)
    mixed = m.pop("tl_precision", None)
    deck = decks.make_deck(x_cells=64, y_cells=64, end_step=1, tl_max_iters=5, **m)
    if mixed:
        deck = deck.replace("*endtea", "tl_precision mixed\n*endtea")
    ch = _chunk(deck)
    info = ch.timestep()
    ch.close()
    assert info["status"] == tl.TL_WARN_MAXITER
    if not mixed:
        assert info["error_ratio"] > 1e-15  # stopped short of tl_eps
    # (mixed CG: tl_max_iters bounds each FP32 inner solve; the FP64
    # refinement around the capped inner solves may still reach tl_eps)


@pytest.mark.parametrize("method", [
    {"tl_use_cg": True, "tl_preconditioner_type": "jac_diag"},
    {"tl_use_cg": False, "tl_use_chebyshev": True, "tl_ch_cg_presteps": 10, "tl_ch_cg_epslim": 1e10},
    {"tl_use_cg": False, "tl_use_ppcg": True, "tl_ppcg_inner_steps": 10,
     "tl_preconditioner_type": "jac_block", "tl_ch_cg_presteps": 10, "tl_ch_cg_epslim": 1e10},
    {"tl_use_cg": False, "tl_use_ppcg": True, "tl_ppcg_inner_steps": 10,
     "tl_preconditioner_type": "jac_block", "tl_ch_cg_presteps": 10, "tl_ch_cg_epslim": 1e10,
     "tl_precision": "mixed"},
    {"tl_use_cg": True, "tl_preconditioner_type": "jac_diag", "tl_precision": "mixed"},
])
def test_nan_in_the_data_stops_with_breakdown(method):
    m = dict(method)
    mixed = m.pop("tl_precision", None)
    deck = decks.make_deck(x_cells=64, y_cells=48, end_step=1, **m)
    if mixed:
        deck = deck.replace("*endtea", "tl_precision mixed\n*endtea")
    ch = _chunk(deck)
    e = ch.get_field("energy1")
    e[20, 30] = np.nan
    ch.set_field("energy1", e)
    with pytest.raises(tl.TeaLeafError) as err:
        ch.timestep()
    assert err.value.code == tl.TL_ERR_BREAKDOWN
    assert "breakdown" in tl.last_error()
    # the context and the chunk stay usable: a restart solves normally
    ch.start()
    info = ch.timestep()
    assert info["status"] == tl.TL_OK
    plain = _chunk(deck)
    ref = plain.timestep()
    assert info["iterations"] == ref["iterations"]
    assert ch.field_summary() == plain.field_summary()
    ch.close()
    plain.close()


def _free_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def test_failed_chunk_allocation_frees_what_it_took():
    lib = tl.load()
    cfg = tl.parse_deck(decks.make_deck(x_cells=512, y_cells=512, end_step=1))
    before = _free_bytes()
    # the chunk makes about 33 device allocations: fail the first, some in
    # the middle and the last ones
    for nth in (1, 2, 7, 21, 22, 28, 31, 33):
        h = C.c_void_p()
        assert lib.tl_test_fail_alloc(nth) == 0
        rc = lib.tl_chunk_create(C.byref(cfg), C.byref(h))
        lib.tl_test_fail_alloc(0)
        if rc == tl.TL_OK:  # fewer allocations than nth: nothing failed
            lib.tl_chunk_destroy(h)
            continue
        assert rc == tl.TL_ERR_ALLOC, (nth, rc, tl.last_error())
        assert "cudaMalloc" in tl.last_error() or "memory" in tl.last_error()
        assert not h.value
        assert before - _free_bytes() < 2 * MIB, nth  # nothing leaked
    ch = tl.Chunk(cfg)
    ch.start()
    assert ch.timestep()["status"] == tl.TL_OK
    ch.close()


@pytest.mark.parametrize("extra", ["tl_precision mixed\ntl_use_ppcg\ntl_ppcg_inner_steps 10\n"
                                   "tl_preconditioner_type jac_block\n",
                                   "tl_warm_start prev\n"])
def test_failed_lazy_allocation_is_retried(extra):
    """The mixed-precision and warm-start buffers are made on the first solve
    that needs them; a failure there leaves no half-made state behind, so
    the next solve allocates again and gives the answer of a fresh chunk."""
    lib = tl.load()
    deck = decks.make_deck(x_cells=96, y_cells=72, end_step=1).replace("*endtea", extra + "*endtea")
    deck = deck.replace("tl_use_cg\n", "") if "ppcg" in extra else deck
    ch = _chunk(deck)
    for nth in (1, 3):
        assert lib.tl_test_fail_alloc(nth) == 0
        with pytest.raises(tl.TeaLeafError) as err:
            ch.timestep()
        lib.tl_test_fail_alloc(0)
        assert err.value.code == tl.TL_ERR_ALLOC
        ch.start()
    info = ch.timestep()
    fresh = _chunk(deck)
    ref = fresh.timestep()
    assert info["status"] == ref["status"] == tl.TL_OK
    assert info["iterations"] == ref["iterations"]
    assert ch.field_summary() == fresh.field_summary()
    ch.close()
    fresh.close()
