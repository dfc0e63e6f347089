"""bench.py on the CPU: its decks parse, and the reference arm (the oracle
on the host cores) prints one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys

import tealeaf_cuda_gb300 as tl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_bench_decks_parse():
    cfg = tl.parse_deck(bench.make_deck(8192, solver="ppcg", precond="jac_block", precision="mixed",
                                        warm="learned"))
    assert (cfg.x_cells, cfg.y_cells) == (8192, 8192)
    assert cfg.solver == tl.SOLVER_PPCG and cfg.precond == tl.PREC_JAC_BLOCK
    assert cfg.precision == tl.PRECISION_MIXED and cfg.warm_start == tl.WARM_LEARNED
    assert cfg.ppcg_inner_steps == 10 and cfg.eps == 1e-15 and cfg.max_iters == 10000
    cfg = tl.parse_deck(bench.make_deck(64))
    assert cfg.solver == tl.SOLVER_CG and cfg.precond == tl.PREC_JAC_DIAG
    assert cfg.precision == tl.PRECISION_FP64 and cfg.warm_start == tl.WARM_NONE
    assert bench.bytes_per_cell("mixed_pp_step", "jac_block") == 40
    assert bench.bytes_per_cell("cg_w", "jac_diag") == 32


def test_bench_fused_pass_bytes():
    """The fused inner passes' byte figure is the mean over one solve's
    passes: a full pass reads sd, rtemp, utemp (12 B) and the coefficients
    and writes sd, rtemp, utemp (12 B); the first reads r (FP64, 8 B)
    instead of sd, rtemp, utemp and the last writes z (FP64, 8 B) instead of
    them."""
    assert bench.INNER_STEPS == 10 and bench.FUSED_STEPS == 5
    coef = {"none": 8, "jac_diag": 12, "jac_block": 16}
    for pc, c in coef.items():
        first = 8 + c + 12
        last = 12 + c + 8
        assert bench.bytes_per_cell("mixed_pp_fused", pc) == (first + last) / 2, pc
    # the outer pass then updates r alone, and u moves into the p pass
    assert bench.bytes_per_cell("mixed_pp_ur", "jac_block") == 24
    assert bench.bytes_per_cell("ppcg_up", "jac_block") == 40


def test_reference_arm_prints_contract_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "64",
                          "--steps", "2", "--warmup", "1", "--ref-iters", "20"],
                         check=True, capture_output=True, text=True, env=env, timeout=300).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["unit"] == d["unit"]
