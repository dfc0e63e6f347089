"""Deck helpers for the tests: write tea.in decks from parameter dicts and
load the golden benchmark fixtures (tests/golden/benchmarks.json)."""
import json
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "benchmarks.json")

# the standard five-state problem on a 10 x 10 domain (BASELINE configs)
STANDARD_STATES = [
    {"index": 1, "density": 100.0, "energy": 0.0001},
    {"index": 2, "density": 0.1, "energy": 25.0, "geometry": "rectangle",
     "xmin": 0.0, "xmax": 1.0, "ymin": 1.0, "ymax": 2.0},
    {"index": 3, "density": 0.1, "energy": 0.1, "geometry": "rectangle",
     "xmin": 1.0, "xmax": 6.0, "ymin": 1.0, "ymax": 2.0},
    {"index": 4, "density": 0.1, "energy": 0.1, "geometry": "rectangle",
     "xmin": 5.0, "xmax": 6.0, "ymin": 1.0, "ymax": 8.0},
    {"index": 5, "density": 0.1, "energy": 0.1, "geometry": "rectangle",
     "xmin": 5.0, "xmax": 10.0, "ymin": 7.0, "ymax": 8.0},
]


def golden():
    with open(GOLDEN) as f:
        return json.load(f)["benchmarks"]


def _fmt(v):
    if isinstance(v, bool):
        return ""
    if isinstance(v, float):
        return repr(v)
    return str(v)


def make_deck(n=None, states=None, **kw):
    """A tea.in deck.  Keyword flags with value True are written bare
    (tl_use_cg), other keywords as `key=value`."""
    params = {"xmin": 0.0, "ymin": 0.0, "xmax": 10.0, "ymax": 10.0,
              "initial_timestep": 0.004, "end_step": 10, "tl_max_iters": 10000,
              "tl_use_cg": True, "tl_eps": 1.0e-15, "halo_depth": 1}
    if n is not None:
        params["x_cells"] = n
        params["y_cells"] = n
    params.update(kw)
    lines = ["*tea"]
    for st in (states or STANDARD_STATES):
        parts = [f"state {st['index']}", f"density={st['density']!r}", f"energy={st['energy']!r}"]
        if "geometry" in st:
            parts.append(f"geometry={st['geometry']}")
            for k in ("xmin", "xmax", "ymin", "ymax", "radius"):
                if k in st:
                    parts.append(f"{k}={st[k]!r}")
        lines.append(" ".join(parts))
    for k, v in params.items():
        if v is False or v is None:
            continue
        if v is True:
            lines.append(k)
        else:
            lines.append(f"{k}={_fmt(v)}")
    lines.append("*endtea")
    return "\n".join(lines) + "\n"


def golden_deck(name):
    d = dict(golden()[name]["deck"])
    states = d.pop("states")
    for k in ("test_problem", "profiler_on"):
        d.pop(k, None)
    return make_deck(states=states, **d)
