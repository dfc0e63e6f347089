"""Build and run the CPU oracle (oracle/) for the tests.  The oracle is the
checker only; nothing here is used by the product."""
import json
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BIN = os.path.join(ORACLE_DIR, "_build", "tea_oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libtea_oracle.so")


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_BIN


def run_deck(deck_text, max_steps=None, threads=None, u_samples=0):
    """Run a deck through the oracle; returns (step records, run record).
    With u_samples S every step record also holds u at an S x S lattice of
    interior cells (`u_samples`, see sample_cells)."""
    build_oracle()
    with tempfile.NamedTemporaryFile("w", suffix=".in", delete=False) as f:
        f.write(deck_text)
        path = f.name
    try:
        cmd = [ORACLE_BIN, path]
        if max_steps:
            cmd += ["--max-steps", str(max_steps)]
        if u_samples:
            cmd += ["--u-samples", str(u_samples)]
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        out = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env).stdout
    finally:
        os.unlink(path)
    recs = [json.loads(l) for l in out.splitlines() if l.strip()]
    steps = [r for r in recs if r["kind"] == "step"]
    run = [r for r in recs if r["kind"] == "run"][0]
    return steps, run


def sample_cells(n, s):
    """0-based interior indices of the oracle's --u-samples lattice along an
    axis of n cells: the centres of an even partition into s parts."""
    return [((2 * k + 1) * n) // (2 * s) for k in range(s)]
