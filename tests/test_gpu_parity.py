"""GPU parity tests: the CUDA path through the C-ABI against the CPU oracle and
the reference's golden benchmark outputs.

Bars (the benchmark spec's tolerances): field_summary within 1e-10 relative and
solver iteration counts within +-1 (Chebyshev: +-10, since it only reads its
residual every 10th iteration, tea_solve.f90:277).  Single kernels are
compared bit for bit: the GPU and the oracle evaluate the same fused
multiply-add expressions and differ only in the order of dot-product sums."""
import ctypes as C

import numpy as np
import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks
from tests.oracle_lib import OracleChunk
from tests.oracle_run import run_deck as oracle_run

pytestmark = pytest.mark.gpu

FS_RTOL = 1e-10
SUMMARY_KEYS = ("vol", "mass", "ie", "temp")


def gpu_run(deck, **kw):
    recs, res = tl.run_deck(deck, **kw)
    assert res["status"] == 0, tl.last_error()
    return recs, res


def assert_summary_close(a, b, rtol=FS_RTOL):
    for k in SUMMARY_KEYS:
        assert a[k] == pytest.approx(b[k], rel=rtol), (k, a[k], b[k])


def compare_to_oracle(deck, its_tol=1):
    recs, _ = gpu_run(deck)
    steps, _ = oracle_run(deck)
    assert len(recs) == len(steps)
    for g, o in zip(recs[1:], steps[1:]):
        assert abs(g["iterations"] - o["iterations"]) <= its_tol, (g["step"], g["iterations"], o["iterations"])
        if "temp" in o:
            assert_summary_close(g, o)
    assert_summary_close(recs[-1], steps[-1])
    return recs, steps


# ------------------------------------------------------------ golden vectors

@pytest.mark.parametrize("name", ["tea_bm_1", "tea_bm_2", "tea_bm_3", "tea_bm_4"])
def test_reference_benchmarks(name):
    g = decks.golden()[name]
    recs, res = gpu_run(decks.golden_deck(name))
    its = [r["iterations"] for r in recs[1:]]
    assert all(abs(a - b) <= 1 for a, b in zip(its, g["iterations"])), (its, g["iterations"])
    fin = recs[-1]
    gf = g["summary_final"]
    for k, gk in zip(SUMMARY_KEYS, ("volume", "mass", "energy", "u")):
        assert fin[k] == pytest.approx(gf[gk], rel=FS_RTOL)
    assert abs(100.0 * fin["temp"] / g["qa_temp"] - 100.0) < 0.001


def test_reference_benchmark_legacy_entry_points():
    """The reference-named per-kernel entry points, driven by the host control
    flow of tea_solve.f90, reproduce the golden run too."""
    g = decks.golden()["tea_bm_2"]
    recs, _ = gpu_run(decks.golden_deck("tea_bm_2"), legacy_abi=True)
    assert [r["iterations"] for r in recs[1:]] == g["iterations"]
    assert recs[-1]["temp"] == pytest.approx(g["summary_final"]["u"], rel=FS_RTOL)


# ------------------------------------------------------ solvers vs oracle

SOLVERS = {
    "cg": {"tl_use_cg": True},
    # Chebyshev reads its residual every 10th iteration and, at tl_eps 1e-15,
    # can stagnate right at the threshold on small grids (the oracle sits at
    # 1.4e-15 for 10000 iterations on 64x48); 1e-12 is attainable for both
    "cheby": {"tl_use_cg": False, "tl_use_chebyshev": True, "tl_ch_cg_presteps": 10,
              "tl_ch_cg_epslim": 1.0e10, "tl_eps": 1.0e-12},
    "ppcg": {"tl_use_cg": False, "tl_use_ppcg": True, "tl_ch_cg_presteps": 10,
             "tl_ch_cg_epslim": 1.0e10, "tl_ppcg_inner_steps": 10},
    # the reference's default solver (read_input.f90:88); it takes no
    # preconditioner (tea_leaf_jacobi.cuknl:5-46)
    "jacobi": {"tl_use_cg": False, "tl_use_jacobi": True},
}
PRECONDS = ["none", "jac_diag", "jac_block"]


@pytest.mark.parametrize("solver", list(SOLVERS))
@pytest.mark.parametrize("precond", PRECONDS)
@pytest.mark.parametrize("shape", [(64, 48), (37, 29)])
def test_solver_matches_oracle(solver, precond, shape):
    deck = decks.make_deck(x_cells=shape[0], y_cells=shape[1], end_step=3,
                           tl_preconditioner_type=precond, **SOLVERS[solver])
    compare_to_oracle(deck, its_tol=10 if solver == "cheby" else 1)


@pytest.mark.parametrize("solver", list(SOLVERS))
@pytest.mark.parametrize("precond", PRECONDS)
def test_device_resident_equals_reference_entry_points(solver, precond):
    """tl_timestep (scalars and exit test on the GPU) and the reference-named
    entry points (scalars on the host) run the same kernels on the same
    numbers, so they agree bit for bit."""
    deck = decks.make_deck(x_cells=40, y_cells=36, end_step=3, tl_preconditioner_type=precond,
                           **SOLVERS[solver])
    fast, _ = gpu_run(deck)
    slow, _ = gpu_run(deck, legacy_abi=True)
    assert [r["iterations"] for r in fast] == [r["iterations"] for r in slow]
    for a, b in zip(fast, slow):
        for k in SUMMARY_KEYS:
            assert a[k] == b[k]


def test_config1_512_cg_matches_oracle():
    """Plain FP64 CG, no preconditioner, 512x512, 10 steps, tl_eps 1e-15."""
    deck = decks.make_deck(n=512, end_step=10)
    compare_to_oracle(deck)


@pytest.mark.parametrize("extra", [{"reflective_boundary": True},
                                   {"tl_coefficient_inverse_density": True},
                                   {"tl_check_result": True},
                                   {"halo_depth": 2}])
def test_flags_match_oracle(extra):
    deck = decks.make_deck(x_cells=50, y_cells=44, end_step=2, tl_preconditioner_type="jac_diag", **extra)
    recs, steps = compare_to_oracle(deck)


@pytest.mark.parametrize("solver", ["ppcg", "cheby"])
@pytest.mark.parametrize("extra", [{"reflective_boundary": True},
                                   {"tl_coefficient_inverse_density": True},
                                   {"halo_depth": 2}])
def test_flags_with_chebyshev_and_ppcg_match_oracle(solver, extra):
    """The same flags under the polynomial solvers (halo_depth 2 takes
    PPCG's matrix-powers inner loop, tea_leaf_ppcg.f90:199-221)."""
    deck = decks.make_deck(x_cells=50, y_cells=44, end_step=2, tl_preconditioner_type="jac_diag",
                           **SOLVERS[solver], **extra)
    compare_to_oracle(deck, its_tol=10 if solver == "cheby" else 1)


def test_determinism():
    deck = decks.make_deck(x_cells=96, y_cells=80, end_step=2, tl_preconditioner_type="jac_diag")
    a, _ = gpu_run(deck)
    b, _ = gpu_run(deck)
    for x, y in zip(a, b):
        assert x["iterations"] == y["iterations"]
        for k in SUMMARY_KEYS + ("error_ratio",):
            assert x[k] == y[k]


# ------------------------------------------------ single kernels, bitwise

def _setup(deck):
    lib = tl.load()
    cfg = tl.parse_deck(deck)
    assert lib.tl_default_chunk_init(C.byref(cfg)) == 0, tl.last_error()
    h = lib.tl_default_chunk()
    v = [C.c_double() for _ in range(4)]
    assert lib.tl_start(h, *[C.byref(x) for x in v]) == 0
    ora = OracleChunk(deck)
    shape = (cfg.y_cells + 2 * cfg.halo_depth, cfg.x_cells + 2 * cfg.halo_depth)

    def gf(name):
        a = np.empty(shape, dtype=np.float64)
        assert lib.tl_get_field(h, tl.FIELDS[name], a.ctypes.data) == 0
        return a

    return lib, cfg, ora, shape, gf


def _interior(a, cfg):
    hd = cfg.halo_depth
    return a[hd:hd + cfg.y_cells, hd:hd + cfg.x_cells]


def _same(lib_field, ora_field, cfg, name):
    g, o = _interior(lib_field, cfg), _interior(ora_field, cfg)
    bad = np.argwhere(g != o)
    assert bad.size == 0, f"{name}: {len(bad)} cells differ, first {bad[:3]} {g[tuple(bad[0])]} vs {o[tuple(bad[0])]}"


@pytest.mark.parametrize("precond", PRECONDS)
def test_cg_kernels_bitwise(precond):
    deck = decks.make_deck(x_cells=45, y_cells=30, end_step=1, tl_preconditioner_type=precond)
    lib, cfg, ora, shape, gf = _setup(deck)
    f = lambda n: ora.field(n, shape)
    by = C.byref
    coef, dt = C.c_int(1), C.c_double(0.004)
    rx, ry, orx, ory = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    zero, refl = (C.c_int * 4)(1, 1, 1, 1), C.c_int(0)
    lib.tea_leaf_common_init_kernel_cuda_(by(coef), by(dt), by(rx), by(ry), zero, by(refl))
    ora.common_init(0.004, by(orx), by(ory))
    assert (rx.value, ry.value) == (orx.value, ory.value)
    for n in ("u", "u0"):
        _same(gf(n), f(n), cfg, n)
    hd, nx, ny = cfg.halo_depth, cfg.x_cells, cfg.y_cells
    # face coefficients the operator reads: Kx on x-faces h..nx+h, Ky on y-faces h..ny+h
    assert np.array_equal(gf("kx")[hd:hd + ny, hd:hd + nx + 1], f("kx")[hd:hd + ny, hd:hd + nx + 1])
    assert np.array_equal(gf("ky")[hd:hd + ny + 1, hd:hd + nx], f("ky")[hd:hd + ny + 1, hd:hd + nx])
    lib.tea_leaf_calc_residual_cuda_()
    ora.calc_residual()
    _same(gf("r"), f("r"), cfg, "r")
    one, nrm = C.c_int(1), C.c_double()
    lib.tea_leaf_calc_2norm_kernel_cuda_(by(one), by(nrm))
    assert nrm.value == pytest.approx(ora.calc_2norm(1), rel=1e-13)
    rro = C.c_double()
    lib.tea_leaf_cg_init_kernel_cuda_(by(rro))
    orro = ora.cg_init()
    assert rro.value == pytest.approx(orro, rel=1e-13)
    names = {"none": ["p"], "jac_diag": ["p", "z", "mi"], "jac_block": ["p", "z", "cp", "bfp"]}[precond]
    for n in names:
        _same(gf(n), f(n), cfg, n)
    for it in range(3):
        pw = C.c_double()
        lib.tea_leaf_cg_calc_w_kernel_cuda_(by(pw))
        opw = ora.cg_calc_w()
        _same(gf("w"), f("w"), cfg, "w")
        assert pw.value == pytest.approx(opw, rel=1e-12)
        alpha = C.c_double(orro / opw)
        rrn = C.c_double()
        lib.tea_leaf_cg_calc_ur_kernel_cuda_(by(alpha), by(rrn))
        orrn = ora.cg_calc_ur(alpha.value)
        for n in ["u", "r"] + (["z"] if precond != "none" else []):
            _same(gf(n), f(n), cfg, n)
        assert rrn.value == pytest.approx(orrn, rel=1e-12)
        beta = C.c_double(orrn / orro)
        lib.tea_leaf_cg_calc_p_kernel_cuda_(by(beta))
        ora.cg_calc_p(beta.value)
        _same(gf("p"), f("p"), cfg, "p")
        orro = orrn
    lib.tea_leaf_common_finalise_kernel_cuda_()
    ora.finalise()
    _same(gf("energy1"), f("energy1"), cfg, "energy1")


@pytest.mark.parametrize("precond", PRECONDS)
def test_cheby_ppcg_kernels_bitwise(precond):
    deck = decks.make_deck(x_cells=33, y_cells=26, end_step=1, tl_preconditioner_type=precond)
    lib, cfg, ora, shape, gf = _setup(deck)
    f = lambda n: ora.field(n, shape)
    by = C.byref
    coef, dt = C.c_int(1), C.c_double(0.004)
    rx, ry = C.c_double(), C.c_double()
    zero, refl = (C.c_int * 4)(1, 1, 1, 1), C.c_int(0)
    lib.tea_leaf_common_init_kernel_cuda_(by(coef), by(dt), by(rx), by(ry), zero, by(refl))
    ora.common_init(0.004, by(C.c_double()), by(C.c_double()))
    lib.tea_leaf_calc_residual_cuda_()
    ora.calc_residual()
    rro = C.c_double()
    lib.tea_leaf_cg_init_kernel_cuda_(by(rro))
    ora.cg_init()
    n = 12
    al = (C.c_double * n)(*[0.3 + 0.01 * k for k in range(n)])
    be = (C.c_double * n)(*[0.02 + 0.001 * k for k in range(n)])
    theta = C.c_double(17.5)
    nn = C.c_int(n)
    # Chebyshev: init (+ calc_u) and three iterations
    lib.tea_leaf_cheby_init_kernel_cuda_(al, be, by(nn), by(theta))
    ora.cheby_init(al, be, n, theta.value)
    for name in ("u", "p", "r", "w"):
        _same(gf(name), f(name), cfg, name)
    for st in (1, 2, 3):
        s = C.c_int(st)
        lib.tea_leaf_cheby_iterate_kernel_cuda_(by(s))
        ora.cheby_iterate(st)
        for name in ("u", "p", "r", "w"):
            _same(gf(name), f(name), cfg, name)
    # PPCG: init steps, inner steps, rrn
    lib.tea_leaf_ppcg_init_constants_cuda_(al, be, by(nn))
    ora.ppcg_init_constants(al, be, n)
    for step in (1, 2, 3):
        s, out = C.c_int(step), C.c_double()
        lib.tea_leaf_ppcg_init_kernel_cuda_(by(s), by(out))
        o = ora.ppcg_init(step)
        assert out.value == pytest.approx(o, rel=1e-12, abs=0.0)
        for name in ("p", "z"):
            _same(gf(name), f(name), cfg, name)
    lib.tea_leaf_ppcg_store_r_kernel_cuda_()
    ora.ppcg_store_r()
    lib.tea_leaf_ppcg_init_sd_new_kernel_cuda_(by(theta))
    ora.ppcg_init_sd_new(theta.value)
    nb = (C.c_int * 4)(-1, -1, -1, -1)
    for st in range(1, 5):
        s, bx = C.c_int(st), C.c_int(0)
        lib.tea_leaf_ppcg_inner_kernel_cuda_(by(s), by(bx), nb)
        ora.ppcg_inner(st)
        for name in ("sd", "rtemp", "utemp"):
            _same(gf(name), f(name), cfg, name)
    lib.tea_leaf_ppcg_update_z_kernel_cuda_()
    ora.ppcg_update_z()
    _same(gf("z"), f("z"), cfg, "z")
    rrn = C.c_double()
    lib.tea_leaf_ppcg_calc_rrn_kernel_cuda_(by(rrn))
    assert rrn.value == pytest.approx(ora.ppcg_calc_rrn(), rel=1e-10, abs=1e-300)


def test_field_summary_and_start_match_oracle():
    deck = decks.make_deck(x_cells=70, y_cells=52, end_step=1)
    lib, cfg, ora, shape, gf = _setup(deck)
    for n in ("density", "energy0", "energy1", "u", "u0", "volume"):
        _same(gf(n), ora.field(n, shape), cfg, n)


def test_errors_are_reported_not_fatal():
    lib = tl.load()
    cfg = tl.parse_deck(decks.make_deck(x_cells=16, y_cells=16))
    cfg.x_cells = 0
    h = C.c_void_p()
    assert lib.tl_chunk_create(C.byref(cfg), C.byref(h)) == tl.TL_ERR_ARG
    assert "invalid grid" in tl.last_error()
    lib.cuda_pack_buffers_(None, None, None, None, None)
    assert "single chunk" in tl.last_error()
