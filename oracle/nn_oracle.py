"""CPU oracle of the warm-start network (TEST INFRASTRUCTURE ONLY).

A numpy restatement of the residual network the CUDA kernels of
tealeaf_cuda_gb300/csrc/tl_conv.cu evaluate and train: six 3x3 convolutions
on NHWC tensors with a one-pixel zero halo, GELU (tanh form), residual blocks,
a linear head, the masked MSE loss, and the backward pass.  With quant=True
the tensors are rounded to bfloat16 at the same points as the GPU kernels
(stored activations, pre-activations, output and data gradients, weights);
accumulation is FP64.  With quant=False everything is FP64, which the tests
check against finite differences.

Only tests/ use this file.
"""
import numpy as np

# (cin, coutp, kind) per layer, as tl_warm.cu
LAYERS = [(16, 32, "gelu")] + [(32, 32, "gelu_res")] * 4 + [(32, 16, "head")]
G0, G1 = 0.7978845608028654, 0.044715


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(G0 * (x + G1 * x ** 3)))


def gelu_grad(x):
    th = np.tanh(G0 * (x + G1 * x ** 3))
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * G0 * (1.0 + 3.0 * G1 * x * x)


def split_params(p):
    """flat FP32 parameters -> [(W [9][coutp][cin], b [coutp])]"""
    out, off = [], 0
    for cin, co, _ in LAYERS:
        n = 9 * co * cin
        out.append((p[off:off + n].reshape(9, co, cin).astype(np.float64),
                    p[off + n:off + n + co].astype(np.float64)))
        off += n + co
    return out


def conv(xp, W):
    """xp [B][H+2][W+2][cin] (padded), W [9][cout][cin] -> [B][H][W][cout]"""
    B, Hp, Wp, _ = xp.shape
    H, Wd = Hp - 2, Wp - 2
    out = np.zeros((B, H, Wd, W.shape[1]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        out += xp[:, dy:dy + H, dx:dx + Wd, :] @ W[tap].T
    return out


def pad(x):
    return np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))


def forward(params, x, quant=True):
    """x: padded input [B][H+2][W+2][16]; returns y [B][H][W] and the cache"""
    q = bf16 if quant else (lambda v: v)
    layers = split_params(params)
    h = x
    cache = {"h": [x], "pre": []}
    for (cin, co, kind), (W, b) in zip(LAYERS, layers):
        v = conv(h, q(W)) + b
        if kind == "head":
            y = v[..., 0]
            break
        cache["pre"].append(pad(q(v)))
        g = gelu(v)
        if kind == "gelu_res":
            g = g + h[:, 1:-1, 1:-1, :]
        h = pad(q(g))
        cache["h"].append(h)
    return y, cache


def loss_and_dy(y, t, margin, quant=True):
    B, H, W = y.shape
    m = np.zeros_like(y)
    m[:, margin:H - margin, margin:W - margin] = 1.0
    cnt = m.sum()
    e = (y - t) * m
    dy = 2.0 * e / cnt
    if quant:
        dy = bf16(dy)
    return float((e * e).sum() / cnt), dy


def backward(params, cache, dy, quant=True):
    """dy [B][H][W] -> [(dW, db)] per layer"""
    q = bf16 if quant else (lambda v: v)
    layers = split_params(params)
    grads = [None] * len(LAYERS)
    B, H, W = dy.shape
    d = np.zeros((B, H + 2, W + 2, 16))
    d[:, 1:-1, 1:-1, 0] = dy
    # head: dW = sum dy * h5, dh5 = conv^T(dy, W6)
    hs = cache["h"]
    grads[5] = wgrad(d, hs[5]), d[:, 1:-1, 1:-1, :].sum(axis=(0, 1, 2))
    dh = pad(q(dgrad(d, q(layers[5][0]))))
    for l in range(4, 0, -1):
        dpre = pad(q(dh[:, 1:-1, 1:-1, :] * gelu_grad(cache["pre"][l][:, 1:-1, 1:-1, :])))
        grads[l] = wgrad(dpre, hs[l]), dpre[:, 1:-1, 1:-1, :].sum(axis=(0, 1, 2))
        dh = pad(q(dh[:, 1:-1, 1:-1, :] + dgrad(dpre, q(layers[l][0]))))
    dpre = pad(q(dh[:, 1:-1, 1:-1, :] * gelu_grad(cache["pre"][0][:, 1:-1, 1:-1, :])))
    grads[0] = wgrad(dpre, hs[0]), dpre[:, 1:-1, 1:-1, :].sum(axis=(0, 1, 2))
    return grads


def dgrad(dp, W):
    """data gradient of conv: dp padded [B][H+2][W+2][cout] -> [B][H][W][cin]"""
    Wf = np.stack([W[8 - tap].T for tap in range(9)])  # [9][cin][cout]
    return conv(dp, Wf)


def wgrad(dp, xp):
    """dW[tap][co][ci] = sum_p dp[p][co] x[p + off(tap)][ci]"""
    B, Hp, Wp, co = dp.shape
    H, W = Hp - 2, Wp - 2
    g = dp[:, 1:-1, 1:-1, :].reshape(-1, co)
    out = np.zeros((9, co, xp.shape[-1]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        xs = xp[:, dy:dy + H, dx:dx + W, :].reshape(-1, xp.shape[-1])
        out[tap] = g.T @ xs
    return out
