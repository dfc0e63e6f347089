"""Extract the reference's golden vectors into tests/golden/benchmarks.json.

The reference (UK-MAC/TeaLeaf_CUDA) has no unit tests; its only known answers
are the benchmark runs Benchmarks/tea_bm_{1..6}.out (CG, no preconditioner,
tl_eps 1e-15, 10 steps of the standard five-state deck) and the QA constants
of field_summary.f90:96-101.  This script reads the benchmark decks and
outputs from a reference checkout and records, per benchmark:

  * the deck parameters (grid, timestep, solver settings, states), so the
    tests can write an equivalent deck without the reference present;
  * the per-step "Iteration count" and "Conduction error" lines;
  * the step-0 and final field_summary rows (volume, mass, density, energy, u);
  * the MPI task count of the run and whether it reported PASSED.

Usage (needs the reference checkout, so it runs in the build container only):
    python tests/golden/make_golden.py /path/to/TeaLeaf_CUDA
"""
import json
import re
import sys
from pathlib import Path

# field_summary.f90:96-101, the expected final temp of test problems 1..6
QA_TEMP = {1: 157.55084183279294, 2: 106.27221178646569, 3: 99.955877498324000,
           4: 97.277332050749976, 5: 95.462351583362249, 6: 95.174738768320850}


def parse_deck(text):
    deck = {"states": []}
    for raw in text.splitlines():
        line = raw.split("!")[0].strip().lower().replace("=", " ").replace(",", " ")
        if not line or line.startswith("*"):
            continue
        words = line.split()
        if words[0] == "state":
            st = {"index": int(words[1])}
            it = iter(words[2:])
            for k in it:
                v = next(it)
                st[k] = v if k == "geometry" else float(v)
            deck["states"].append(st)
            continue
        key = words[0]
        if len(words) == 1:
            deck[key] = True
        else:
            v = words[1]
            try:
                deck[key] = int(v)
            except ValueError:
                try:
                    deck[key] = float(v)
                except ValueError:
                    deck[key] = v
    return deck


def parse_out(text):
    its = [int(x) for x in re.findall(r"Iteration count\s+(\d+)", text)]
    errs = [float(x) for x in re.findall(r"Conduction error\s+(\S+)", text)]
    rows = []
    for line in text.splitlines():
        s = line.split()
        if s and s[0] == "step:":
            rows.append({"step": int(s[1]), "volume": float(s[2]), "mass": float(s[3]),
                         "density": float(s[4]), "energy": float(s[5]), "u": float(s[6])})
    tasks = re.search(r"Task Count\s+(\d+)", text)
    return {
        "iterations": its,
        "conduction_error": errs,
        "summary_step0": rows[0],
        "summary_final": rows[-1],
        "mpi_tasks": int(tasks.group(1)) if tasks else None,
        "passed": "considered PASSED" in text,
    }


def main(ref):
    bench = Path(ref) / "Benchmarks"
    out = {"source": "Benchmarks/tea_bm_{1..6}.{in,out} and field_summary.f90:96-101",
           "benchmarks": {}}
    for i in range(1, 7):
        deck = parse_deck((bench / f"tea_bm_{i}.in").read_text())
        res = parse_out((bench / f"tea_bm_{i}.out").read_text())
        res["deck"] = deck
        res["qa_temp"] = QA_TEMP[i]
        out["benchmarks"][f"tea_bm_{i}"] = res
    dst = Path(__file__).with_name("benchmarks.json")
    dst.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/TeaLeaf_CUDA")
    main(sys.argv[1])
