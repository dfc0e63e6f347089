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


_DIST_PROBE = r"""
import json, os, sys
sys.path.insert(0, os.environ["TL_ROOT"])
import bench
rank, ws, local = bench.dist_init()
bench.barrier(ws)
mx = bench.allreduce_max(rank + 1.5, ws, local)
sm = bench.allreduce_sum(rank + 1.0, ws, local)
bench.barrier(ws)
print(json.dumps({"rank": rank, "ws": ws, "max": mx, "sum": sm}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_bench_rank_helpers_over_gloo_world_size_2():
    """bench.py's rank set-up, barrier and max / sum over ranks (the timing
    max and the whole-job sum of its N>1 replicas) on two gloo ranks."""
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, TL_ROOT=ROOT, TL_BENCH_GLOO="1", RANK=str(rank), LOCAL_RANK=str(rank),
                   WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", _DIST_PROBE], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err
        outs.append(json.loads([l for l in out.splitlines() if l.startswith("{")][0]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["ws"] == 2 and o["max"] == 2.5 and o["sum"] == 3.0


def test_reference_arm_runs_on_rank_0_only():
    """Under a launcher with two ranks the reference arm's rank 1 exits 0
    without work and prints nothing."""
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "64",
                        "--steps", "1", "--warmup", "1", "--ref-iters", "5"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert not [l for l in r.stdout.splitlines() if l.startswith("{")]
