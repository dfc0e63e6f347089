"""CPU-only checks of the C-ABI library: it loads without a GPU, exports every
function include/tealeaf_capi.h declares, its ctypes mirrors match the C
structs, and its deck reader follows parse.f90 / read_input.f90."""
import ctypes as C
import os
import re

import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tealeaf_capi.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("sizeof",)))


def test_library_exports_every_declared_function():
    lib = tl.load()
    names = declared_functions()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_entry_points_are_all_exported():
    lib = tl.load()
    for name in tl.LEGACY_SIGNATURES:
        assert hasattr(lib, name), name
    # the 29 reference symbols of tea_leaf_kernel_cuda.cu and friends
    assert len(tl.LEGACY_SIGNATURES) == 29


def test_struct_mirrors_match_c():
    lib = tl.load()
    for k, s in enumerate(tl._STRUCTS):
        assert lib.tl_sizeof(k) == C.sizeof(s), s.__name__
    assert lib.tl_sizeof(99) == -1


@pytest.mark.parametrize("name", ["tea_bm_1", "tea_bm_4", "tea_bm_5"])
def test_deck_parser_reads_benchmark_decks(name):
    g = decks.golden()[name]["deck"]
    cfg = tl.parse_deck(decks.golden_deck(name))
    assert cfg.x_cells == g["x_cells"] and cfg.y_cells == g["y_cells"]
    assert cfg.solver == tl.SOLVER_CG
    assert cfg.eps == 1.0e-15
    assert cfg.max_iters == 10000
    assert cfg.dtinit == 0.004
    assert cfg.end_step == 10
    assert cfg.nstates == 5
    dx = 10.0 / g["x_cells"]
    # read_input.f90:320-327: states 2..N shrunk by dx/100
    assert cfg.states[1].xmin == pytest.approx(0.0 + dx / 100.0, rel=0, abs=1e-15)
    assert cfg.states[1].xmax == pytest.approx(1.0 - dx / 100.0, rel=0, abs=1e-15)
    assert cfg.states[0].density == 100.0 and cfg.states[1].energy == 25.0
    assert cfg.states[1].geometry == 1
    # tl_ppcg_inner_steps default: 4*INT(SQRT(SQRT(REAL(x*y))))
    assert cfg.ppcg_inner_steps == 4 * int((g["x_cells"] * g["y_cells"]) ** 0.25)


def test_deck_parser_defaults_and_flags():
    text = ("junk before the section\n*tea\nstate 1 density=1.0 energy=2.0\n"
            "x_cells 20 , y_cells=8 ! comment\nTL_USE_PPCG\ntl_preconditioner_type jac_block\n"
            "tl_ppcg_inner_steps 10 ; more\nreflective_boundary\ntl_check_result\n"
            "tl_coefficient_inverse_density\nhalo_depth=2\ntl_max_iters \\\n 77\n"
            "tl_precision mixed\ntl_inner_eps 1e-5\n*endtea\nx_cells 999\n")
    with pytest.raises(ValueError, match="nonstandard halo depth"):
        tl.parse_deck(text)
    cfg = tl.parse_deck(text.replace("halo_depth=2", "halo_depth=1"))
    assert (cfg.x_cells, cfg.y_cells) == (20, 8)
    assert cfg.solver == tl.SOLVER_PPCG and cfg.precond == tl.PREC_JAC_BLOCK
    assert cfg.ppcg_inner_steps == 10 and cfg.max_iters == 77
    assert cfg.reflective_boundary == 1 and cfg.check_result == 1 and cfg.coefficient == 2
    assert cfg.precision == tl.PRECISION_MIXED and cfg.inner_eps == 1e-5
    assert cfg.eps == 1e-10 and cfg.end_step == 640000 and cfg.summary_frequency == 10
    assert cfg.warm_start == tl.WARM_NONE
    for word, mode in (("none", tl.WARM_NONE), ("prev", tl.WARM_PREV), ("learned", tl.WARM_LEARNED)):
        cfg = tl.parse_deck(text.replace("halo_depth=2", f"tl_warm_start {word}"))
        assert cfg.warm_start == mode
    with pytest.raises(ValueError, match="tl_warm_start"):
        tl.parse_deck(text.replace("halo_depth=2", "tl_warm_start guess"))


@pytest.mark.parametrize("bad,msg", [("*tea\nx_cells 10\n*endtea\n", "No states"),
                                     ("*tea\nstate 1 density=1 energy=1\nx_cells ten\n*endtea\n", "integer"),
                                     ("*tea\nstate 1 density=1 energy=1\ntl_preconditioner_type fancy\n*endtea\n",
                                      "preconditioner"),
                                     ("*tea\nstate 1 density=1 energy=1\nstate 1 density=2\n*endtea\n", "twice")])
def test_deck_errors(bad, msg):
    with pytest.raises(ValueError, match=msg):
        tl.parse_deck(bad)


def test_calls_without_a_chunk_fail_with_status():
    lib = tl.load()
    info = tl.SolveInfo()
    assert lib.tl_timestep(None, C.byref(info)) == tl.TL_ERR_STATE
    assert "no chunk" in tl.last_error()
    # a reference-named entry point with no chunk records an error, no crash
    pw = C.c_double(-1.0)
    if lib.tl_default_chunk() is None:
        lib.tea_leaf_cg_calc_w_kernel_cuda_(C.byref(pw))
        assert "initialise_cuda_" in tl.last_error()
        assert pw.value == -1.0


def test_integration_c_example_compiles_and_links(tmp_path):
    """The C usage shown to integrators (deck text -> config -> chunk ->
    start -> timestep -> field summary) compiles as C11 against the public
    header and links against the library (it is not run: that needs a GPU)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "example.c"
    src.write_text(r'''
#include <stdio.h>
#include "tealeaf_capi.h"
int run(const char *deck_text) {
    tl_config_t cfg; char err[256];
    if (tl_parse_deck(deck_text, &cfg, err, sizeof err) != TL_OK) { fprintf(stderr, "%s\n", err); return 1; }
    tl_chunk_t *ch; if (tl_chunk_create(&cfg, &ch) != TL_OK) return 1;
    double vol, mass, ie, temp; tl_start(ch, &vol, &mass, &ie, &temp);
    tl_solve_info_t info; int rc = tl_timestep(ch, &info);
    tl_field_summary(ch, &vol, &mass, &ie, &temp);
    tl_chunk_destroy(ch);
    return rc < 0;
}
int main(void) { return run("*tea\nstate 1 density=100.0 energy=0.0001\nx_cells=8\ny_cells=8\n*endtea\n"); }
''')
    build = os.path.join(ROOT, "tealeaf_cuda_gb300", "_build")
    out = tmp_path / "example"
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", build, "-ltealeaf_gb300", "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_alloc_failure_hook_checks_its_argument():
    """tl_test_fail_alloc only arms a counter on the host (no GPU call)."""
    lib = tl.load()
    assert lib.tl_test_fail_alloc(-1) == tl.TL_ERR_ARG
    assert "nth" in tl.last_error()
    assert lib.tl_test_fail_alloc(0) == tl.TL_OK
