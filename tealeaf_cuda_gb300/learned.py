"""Learned warm start: seeded random decks, trajectory data from the solver,
the trainer of the residual network on the project's own BF16 tensor-core
kernels (tl_nn_* in csrc/tl_conv.cu), model files, and the evaluation of
what the warm starts save over the plain start.

Network (tl_warm.cu): it corrects the start that the last increments give
alone, u_h; inputs (u^n / max|u^n|, log density, log1p Kx, log1p Ky,
100 dt, r_h / max|r_h|, d_1 / max|r_h|) with r_h = u^n - A u_h and
d_1 = u^n - u^{n-1}; six 3x3 convolutions of 32 channels (GELU, four
residual blocks); output (u^{n+1} - u_h) / max|r_h|.  The solve starts from
u^n plus the energy-minimising combination of the network's output and the
last eight increments, and keeps tl_eps * (plain start residual) as its exit
test.  Torch only allocates
device buffers here; every FLOP of the network runs in the library's
kernels.
"""
import ctypes as C
import math
import struct

import numpy as np

from . import Chunk, load, parse_deck

LAYERS = [(16, 32, 0)] + [(32, 32, 1)] * 4 + [(32, 16, 2)]  # (cin, coutp, conv mode)
NFEAT = 8           # per cell: seven network inputs + the target
WARM = {"none": 0, "learned": 1, "prev": 2}  # TL_WARM_*
MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014), the counter-based generator of the decks."""

    def __init__(self, seed):
        self.state = seed & MASK64

    def next(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, a=0.0, b=1.0):
        return a + (b - a) * (self.next() >> 11) / float(1 << 53)

    def log_uniform(self, a, b):
        return math.exp(self.uniform(math.log(a), math.log(b)))

    def randint(self, n):
        return self.next() % n


def random_states(seed):
    """3-8 axis-aligned rectangles of density U[0.05, 200] and energy
    log-uniform [1e-4, 50] over a background drawn the same way."""
    rng = SplitMix64(seed)
    states = [{"index": 1, "density": rng.uniform(0.05, 200.0), "energy": rng.log_uniform(1e-4, 50.0)}]
    for k in range(3 + rng.randint(6)):
        x0, x1 = sorted((rng.uniform(0.0, 10.0), rng.uniform(0.0, 10.0)))
        y0, y1 = sorted((rng.uniform(0.0, 10.0), rng.uniform(0.0, 10.0)))
        x1, y1 = max(x1, x0 + 0.3), max(y1, y0 + 0.3)
        states.append({"index": k + 2, "density": rng.uniform(0.05, 200.0),
                       "energy": rng.log_uniform(1e-4, 50.0), "geometry": "rectangle",
                       "xmin": x0, "xmax": x1, "ymin": y0, "ymax": y1})
    return states


def deck_text(states, n, steps, precond="jac_diag", eps=1e-15, extra=None):
    """A tea.in deck.  The reader keeps only the first 100 characters of a
    line (parse.f90:132, FMT='(a100)'), so each state is split over lines
    joined by the parser's `\\` continuation."""
    lines = ["*tea"]
    for st in states:
        lines.append(f"state {st['index']} density={st['density']!r} energy={st['energy']!r}" +
                     (" \\" if "geometry" in st else ""))
        if "geometry" in st:
            lines.append(f"  geometry={st['geometry']} xmin={st['xmin']!r} xmax={st['xmax']!r} \\")
            lines.append(f"  ymin={st['ymin']!r} ymax={st['ymax']!r}")
    assert all(len(l) <= 100 for l in lines)
    lines += [f"x_cells={n}", f"y_cells={n}", "xmin=0.0", "ymin=0.0", "xmax=10.0", "ymax=10.0",
              "initial_timestep=0.004", f"end_step={steps}", "tl_max_iters=10000", "tl_use_cg",
              f"tl_preconditioner_type {precond}", f"tl_eps {eps!r}", "summary_frequency 0"]
    lines += list(extra or [])
    lines.append("*endtea")
    return "\n".join(lines) + "\n"


def random_deck(seed, n, steps, **kw):
    return deck_text(random_states(seed), n, steps, **kw)


# the five-state problem of the reference's benchmark decks (tea_bm_*.in)
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


def deck_for(spec, n, steps, **kw):
    """"standard" (the benchmark deck) or a random deck's seed"""
    if spec == "standard":
        return deck_text(STANDARD_STATES, n, steps, **kw)
    return random_deck(int(spec), n, steps, **kw)


def parse_decks(text):
    """"standard,20000-20019" -> ["standard", 20000, ..., 20019]"""
    out = []
    for part in text.split(","):
        if part == "standard":
            out.append(part)
        elif "-" in part:
            lo, hi = (int(x) for x in part.split("-"))
            out += list(range(lo, hi + 1))
        else:
            out.append(int(part))
    return out


# algorithmic HBM bytes per cell of one outer iteration of the headline
# method's PPCG phase (mixed precision, two fused passes of 5 inner steps):
# w = Ap with p.w, r.z and r_store (64), rrn (24), u and p (40), r (24),
# and the two fused passes (36 each)
PPCG_OUTER_BYTES_PER_CELL = 64 + 24 + 40 + 24 + 2 * 36


# ---------------------------------------------------------------- model

def param_count():
    return sum(9 * cin * co + co for cin, co, _ in LAYERS)


def init_params(seed=0, head_scale=0.05):
    rng = np.random.default_rng(seed)
    out = []
    for li, (cin, co, _) in enumerate(LAYERS):
        cin_eff = 5 if li == 0 else cin
        W = np.zeros((9, co, cin), dtype=np.float32)
        std = math.sqrt(2.0 / (9 * cin_eff))
        if li == len(LAYERS) - 1:
            W[:, 0, :] = rng.normal(0.0, std * head_scale, (9, cin))
        else:
            W[:, :, :cin_eff] = rng.normal(0.0, std, (9, co, cin_eff))
        out += [W.ravel(), np.zeros(co, dtype=np.float32)]
    p = np.concatenate(out).astype(np.float32)
    assert p.size == param_count()
    return p


def save_model(path, params):
    p = np.ascontiguousarray(params, dtype=np.float32)
    with open(path, "wb") as f:
        f.write(b"TLWS0001")
        f.write(struct.pack("<q", p.size))
        f.write(p.tobytes())


def load_model(path):
    with open(path, "rb") as f:
        assert f.read(8) == b"TLWS0001", "not a warm start model"
        (n,) = struct.unpack("<q", f.read(8))
        return np.frombuffer(f.read(4 * n), dtype=np.float32).copy()


# ----------------------------------------------------------------- data

def trajectories(seeds, n, steps, device="cuda:0", precond="jac_diag"):
    """Solve `steps` timesteps of each seeded deck (FP64, increment-history
    warm start, which tracks the increments) and keep, per step,
    [n][n][NFEAT] = (network inputs of step n, (u^{n+1} - u_h) / max|r_h|)."""
    import torch
    lib = load()
    data = torch.empty((len(seeds) * steps, n, n, NFEAT), dtype=torch.float32, device=device)
    iters = []
    k = 0
    for seed in seeds:
        cfg = parse_deck(random_deck(seed, n, steps, precond=precond))
        cfg.warm_start = WARM["prev"]
        with Chunk(cfg) as ch:
            ch.start()
            for _ in range(steps):
                info = ch.timestep()
                iters.append(info["iterations"])
                rc = lib.tl_warm_start_features(ch._h, C.c_void_p(data[k].data_ptr()))
                assert rc == 0
                k += 1
    torch.cuda.synchronize()
    return data, iters


def trajectory_crops(seeds, n, steps, crops_per_step, crop=144, seed=0, device="cuda:0",
                     precond="jac_diag", every=1):
    """Like trajectories(), but keeps `crops_per_step` random crop x crop
    windows of every `every`-th step instead of whole fields (a 3x3-conv
    network is translation-equivariant, so crops are enough to train it and
    keep large grids in memory).  Returns ([N][crop][crop][NFEAT], iterations)."""
    import torch
    lib = load()
    rng = np.random.default_rng(seed)
    kept = sum(1 for s in range(steps) if s % every == 0)
    data = torch.empty((len(seeds) * kept * crops_per_step, crop, crop, NFEAT), dtype=torch.float32,
                       device=device)
    full = torch.empty((n, n, NFEAT), dtype=torch.float32, device=device)
    iters = []
    k = 0
    for sd in seeds:
        cfg = parse_deck(random_deck(sd, n, steps, precond=precond))
        cfg.warm_start = WARM["prev"]
        with Chunk(cfg) as ch:
            ch.start()
            for s in range(steps):
                info = ch.timestep()
                iters.append(info["iterations"])
                if s % every:
                    continue
                assert lib.tl_warm_start_features(ch._h, C.c_void_p(full.data_ptr())) == 0
                for _ in range(crops_per_step):
                    y0, x0 = rng.integers(0, n - crop + 1, 2)
                    data[k].copy_(full[y0:y0 + crop, x0:x0 + crop])
                    k += 1
    torch.cuda.synchronize()
    return data, iters


# -------------------------------------------------------------- trainer

def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class Trainer:
    """Adam on FP32 master weights; forward and backward on tl_nn_* kernels
    with BF16 activations and FP32 accumulation."""

    def __init__(self, params, batch=16, crop=144, margin=8, lr=1e-3, device="cuda:0"):
        import torch
        self.torch = torch
        self.lib = load()
        self.B, self.S, self.margin, self.lr = batch, crop, margin, lr
        self.dev = device
        B, S = batch, crop
        f32 = dict(dtype=torch.float32, device=device)
        b16 = dict(dtype=torch.bfloat16, device=device)
        self.params = torch.tensor(params, **f32)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.views = []  # (W, b, dW, db, wf, wb) per layer
        off = 0
        for cin, co, _ in LAYERS:
            nw = 9 * cin * co
            self.views.append((self.params[off:off + nw], self.params[off + nw:off + nw + co],
                               self.grad[off:off + nw], self.grad[off + nw:off + nw + co],
                               torch.zeros(nw, **b16), torch.zeros(nw, **b16)))
            off += nw + co
        P = (B, S + 2, S + 2)
        self.x = torch.zeros(P + (16,), **b16)
        self.h = [torch.zeros(P + (32,), **b16) for _ in range(6)]
        self.pre = [torch.zeros(P + (32,), **b16) for _ in range(5)]
        self.y = torch.zeros((B, S, S), **f32)
        self.t = torch.zeros((B, S, S), **f32)
        self.dy = torch.zeros(P + (16,), **b16)
        self.dh = [torch.zeros(P + (32,), **b16) for _ in range(2)]
        self.dpre = torch.zeros(P + (32,), **b16)
        self.gpc = 8
        nmax = max(self.lib.tl_nn_wgrad_partial_floats(cin, co, B, S, S, self.gpc) for cin, co, _ in LAYERS)
        self.partial = torch.zeros(int(nmax), **f32)
        self.loss_part = torch.zeros(1216, **f32)
        self.org = torch.zeros((B, 3), dtype=torch.int32, device=device)
        self.step_no = 0
        self.stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.pack()

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {self.lib.tl_last_error().decode()}")

    def pack(self):
        for (W, b, dW, db, wf, wb), (cin, co, _) in zip(self.views, LAYERS):
            self.check(self.lib.tl_nn_pack(_p(W), _p(wf), _p(wb), cin, co, self.stream), "pack")

    def forward(self):
        L, B, S, s = self.lib, self.B, self.S, self.stream
        hin = self.x
        for li, (cin, co, mode) in enumerate(LAYERS):
            W, b, dW, db, wf, wb = self.views[li]
            if mode == 2:
                self.check(L.tl_nn_conv(2, cin, co, _p(hin), _p(wf), _p(b), None, None, None, _p(self.y),
                                        B, S, S, s), "head")
            else:
                out = self.h[li]
                res = hin if mode == 1 else None
                self.check(L.tl_nn_conv(mode, cin, co, _p(hin), _p(wf), _p(b), _p(res), _p(out),
                                        _p(self.pre[li]), None, B, S, S, s), "conv")
                hin = out
        return self.y

    def backward(self):
        L, B, S, s = self.lib, self.B, self.S, self.stream
        # head
        W, b, dW, db, wf, wb = self.views[5]
        self.check(L.tl_nn_wgrad(_p(self.dy), _p(self.h[4]), 32, 16, _p(self.partial), _p(dW), _p(db),
                                 B, S, S, self.gpc, s), "wgrad head")
        dh = self.dh[0]
        self.check(L.tl_nn_conv(3, 16, 32, _p(self.dy), _p(wb), None, None, _p(dh), None, None, B, S, S, s),
                   "dgrad head")
        for li in range(4, 0, -1):
            W, b, dW, db, wf, wb = self.views[li]
            self.check(L.tl_nn_gelu_backward(_p(dh), _p(self.pre[li]), _p(self.dpre), 32, B, S, S, s), "gelu'")
            self.check(L.tl_nn_wgrad(_p(self.dpre), _p(self.h[li - 1]), 32, 32, _p(self.partial), _p(dW),
                                     _p(db), B, S, S, self.gpc, s), "wgrad")
            dn = self.dh[1] if dh is self.dh[0] else self.dh[0]
            self.check(L.tl_nn_conv(3, 32, 32, _p(self.dpre), _p(wb), None, _p(dh), _p(dn), None, None,
                                    B, S, S, s), "dgrad")
            dh = dn
        W, b, dW, db, wf, wb = self.views[0]
        self.check(L.tl_nn_gelu_backward(_p(dh), _p(self.pre[0]), _p(self.dpre), 32, B, S, S, s), "gelu'")
        self.check(L.tl_nn_wgrad(_p(self.dpre), _p(self.x), 16, 32, _p(self.partial), _p(dW), _p(db),
                                 B, S, S, self.gpc, s), "wgrad 1")

    def loss(self):
        """dy of the masked MSE; per-CTA partial sums of the squared error
        land in loss_part (region_mse() reads them)"""
        L = self.lib
        self.check(L.tl_nn_loss(_p(self.y), _p(self.t), _p(self.dy), _p(self.loss_part), 16, self.B, self.S,
                                self.S, self.margin, self.stream), "loss")

    def step(self, data, rng):
        """one Adam step on a batch of random crops of `data` ([N][H][W][NFEAT])"""
        torch = self.torch
        N, H, W, F = data.shape
        S = self.S
        org = np.stack([rng.integers(0, N, self.B), rng.integers(0, H - S + 1, self.B),
                        rng.integers(0, W - S + 1, self.B)], axis=1).astype(np.int32)
        self.org.copy_(torch.from_numpy(org))
        self.check(self.lib.tl_nn_gather(_p(data), _p(self.org), _p(self.x), _p(self.t), F, 16, H, W, self.B,
                                         S, self.stream), "gather")
        self.forward()
        self.loss()
        self.backward()
        self.step_no += 1
        self.check(self.lib.tl_nn_adam(_p(self.params), _p(self.grad), _p(self.m), _p(self.v),
                                       self.params.numel(), self.lr, 0.9, 0.999, 1e-8, self.step_no,
                                       self.stream), "adam")
        self.pack()

    def region_mse(self):
        cnt = self.B * (self.S - 2 * self.margin) ** 2
        return float(self.loss_part.sum().item()) / cnt

    def params_host(self):
        return self.params.detach().cpu().numpy().copy()


def train(data, iters=1500, batch=16, crop=144, lr=2e-3, seed=0, init=None, log_every=0):
    """Train on trajectory data; returns (params, loss history)."""
    params = init if init is not None else init_params(seed)
    tr = Trainer(params, batch=batch, crop=crop, lr=lr, device=str(data.device))
    rng = np.random.default_rng(seed)
    hist = []
    for it in range(iters):
        tr.step(data, rng)
        if log_every and (it % log_every == 0 or it == iters - 1):
            hist.append((it, tr.region_mse()))
    return tr.params_host(), hist


# ------------------------------------------------------------ evaluation

def solve_with(mode, params, deck, steps, precision=None):
    """Per-step solve info of a deck with warm start `mode` ("none", "prev"
    or "learned"; params = the model of "learned")."""
    lib = load()
    cfg = parse_deck(deck)
    cfg.warm_start = WARM[mode]
    if precision is not None:
        cfg.precision = precision
    out = []
    with Chunk(cfg) as ch:
        ch.start()
        if mode == "learned":
            p = np.ascontiguousarray(params, dtype=np.float32)
            assert lib.tl_set_warm_start_model(ch._h, C.c_void_p(p.ctypes.data), p.size) == 0
        for _ in range(steps):
            info = ch.timestep()
            info["summary"] = ch.field_summary()
            out.append(info)
    return out


def evaluate(params, seeds, n, steps, precond="jac_diag"):
    """Iterations of the plain, previous-step and learned starts on held-out decks."""
    rows = []
    for seed in seeds:
        deck = random_deck(seed, n, steps, precond=precond)
        runs = {m: solve_with(m, params, deck, steps) for m in ("none", "prev", "learned")}
        plain = runs["none"]
        row = {"seed": seed}
        for m, r in runs.items():
            row[m + "_iters"] = [x["iterations"] for x in r]
            row[m + "_seconds"] = sum(x["seconds"] for x in r)
            row[m + "_ratio"] = [x["warm_ratio"] for x in r]
            row[m + "_summary_rel_diff"] = max(abs(a - b) / abs(a) for a, b in
                                               zip(plain[-1]["summary"], r[-1]["summary"]))
        rows.append(row)
    return rows


def compare_methods(params, seeds, n, steps, warm="learned"):
    """Plain FP64 CG + jac_diag from u = u^n against the headline method
    (PPCG + block-Jacobi, 10 FP32 inner steps under the FP64 outer solve,
    warm start `warm`) on the given decks ("standard" or a random deck's
    seed): per timestep the iterations (outer, and PPCG inner), the solve's
    wall time and the field summaries' relative difference."""
    from . import PREC_JAC_BLOCK, PRECISION_MIXED, SOLVER_PPCG
    lib = load()
    rows = []
    for seed in seeds:
        deck = deck_for(seed, n, steps)
        out = {}
        for name in ("plain", "headline"):
            cfg = parse_deck(deck)
            if name == "headline":
                cfg.solver = SOLVER_PPCG
                cfg.precond = PREC_JAC_BLOCK
                cfg.ppcg_inner_steps = 10
                cfg.precision = PRECISION_MIXED
                cfg.warm_start = WARM[warm]
            recs = []
            with Chunk(cfg) as ch:
                ch.start()
                if name == "headline" and warm == "learned":
                    p = np.ascontiguousarray(params, dtype=np.float32)
                    assert lib.tl_set_warm_start_model(ch._h, C.c_void_p(p.ctypes.data), p.size) == 0
                for _ in range(steps):
                    info = ch.timestep()
                    assert info["status"] == 0, (seed, name, info["status"])
                    recs.append((info["iterations"], info["seconds"], ch.field_summary(),
                                 info["ppcg_inner_iters"]))
            out[name] = recs
        hs = [r[1] for r in out["headline"]]
        outer = [r[0] for r in out["headline"]]
        rows.append({"seed": seed,
                     "plain_iters": [r[0] for r in out["plain"]],
                     "headline_iters": outer,
                     "headline_inner_iters": [r[3] for r in out["headline"]],
                     "plain_seconds": [r[1] for r in out["plain"]],
                     "headline_seconds": hs,
                     "headline_hbm_gbs_estimate": n * n * sum(outer) * PPCG_OUTER_BYTES_PER_CELL / sum(hs) / 1e9,
                     "summary_rel_diff": [max(abs(a - b) / abs(b) for a, b in zip(h[2], q[2]))
                                          for h, q in zip(out["headline"], out["plain"])]})
    return rows


def summarise(rows):
    """totals of evaluate()'s rows"""
    out = {}
    for m in ("none", "prev", "learned"):
        out[m + "_iterations"] = sum(sum(r[m + "_iters"]) for r in rows)
        out[m + "_seconds"] = sum(r[m + "_seconds"] for r in rows)
        out[m + "_max_summary_rel_diff"] = max(r[m + "_summary_rel_diff"] for r in rows)
    out["solves"] = sum(len(r["none_iters"]) for r in rows)
    return out


def main(argv=None):
    """python -m tealeaf_cuda_gb300.learned train|evaluate|compare ...

    train:    trajectories of seeded random decks -> model file (+ JSON report)
    evaluate: plain vs previous-step vs learned start on held-out seeds
    compare:  plain FP64 CG against the headline method on held-out seeds"""
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(prog="python -m tealeaf_cuda_gb300.learned")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--decks", type=int, default=200)
    t.add_argument("--first-seed", type=int, default=0)
    t.add_argument("--steps", type=int, default=30)
    t.add_argument("--every", type=int, default=1)
    t.add_argument("--n", type=int, default=2048)
    t.add_argument("--crops", type=int, default=4)
    t.add_argument("--iters", type=int, default=3000)
    t.add_argument("--batch", type=int, default=32)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--out", required=True)
    t.add_argument("--report", default=None)
    e = sub.add_parser("evaluate")
    e.add_argument("--model", required=True)
    e.add_argument("--seeds", default="10000-10049")
    e.add_argument("--n", type=int, default=2048)
    e.add_argument("--steps", type=int, default=3)
    e.add_argument("--report", default=None)
    m = sub.add_parser("compare")
    m.add_argument("--model", required=True)
    m.add_argument("--decks", "--seeds", dest="decks", default="20000-20002",
                   help='"standard" and/or seed ranges, e.g. standard,20000-20019')
    m.add_argument("--n", type=int, default=8192)
    m.add_argument("--steps", type=int, default=5)
    m.add_argument("--warm", default="learned", choices=["none", "prev", "learned"])
    m.add_argument("--report", default=None)
    a = ap.parse_args(argv)
    if a.cmd == "compare":
        rows = compare_methods(load_model(a.model), parse_decks(a.decks), a.n, a.steps, warm=a.warm)
        tp = sum(sum(r["plain_seconds"]) for r in rows)
        th = sum(sum(r["headline_seconds"]) for r in rows)
        rep = {"n": a.n, "steps": a.steps, "decks_run": a.decks, "warm": a.warm,
               "plain_seconds": tp, "headline_seconds": th, "speedup": tp / th,
               "plain_iterations": sum(sum(r["plain_iters"]) for r in rows),
               "headline_outer_iterations": sum(sum(r["headline_iters"]) for r in rows),
               "headline_inner_iterations": sum(sum(r["headline_inner_iters"]) for r in rows),
               "max_summary_rel_diff": max(max(r["summary_rel_diff"]) for r in rows),
               "decks": rows}
        print(json.dumps({k: v for k, v in rep.items() if k != "decks"}))
        if a.report:
            json.dump(rep, open(a.report, "w"), indent=1)
        return
    if a.cmd == "train":
        t0 = time.time()
        seeds = list(range(a.first_seed, a.first_seed + a.decks))
        data, iters = trajectory_crops(seeds, a.n, a.steps, a.crops, every=a.every)
        t1 = time.time()
        params, hist = train(data, iters=a.iters, batch=a.batch, lr=a.lr, log_every=max(1, a.iters // 20))
        t2 = time.time()
        save_model(a.out, params)
        rep = {"decks": a.decks, "steps": a.steps, "n": a.n, "samples": int(data.shape[0]),
               "plain_iterations_mean": float(np.mean(iters)), "data_seconds": t1 - t0,
               "train_seconds": t2 - t1, "loss": hist}
        print(json.dumps(rep))
        if a.report:
            json.dump(rep, open(a.report, "w"), indent=1)
    else:
        lo, hi = (int(x) for x in a.seeds.split("-"))
        rows = evaluate(load_model(a.model), list(range(lo, hi + 1)), a.n, a.steps)
        rep = {"n": a.n, "steps": a.steps, "seeds": a.seeds, **summarise(rows), "decks": rows}
        print(json.dumps({k: v for k, v in rep.items() if k != "decks"}))
        if a.report:
            json.dump(rep, open(a.report, "w"), indent=1)


if __name__ == "__main__":
    main()
