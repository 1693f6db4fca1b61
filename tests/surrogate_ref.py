"""Plain PyTorch FP32 reference of the surrogate MLP (test helper): the same parameter layout as
the library (bude_surrogate_params), BF16 rounding at the points the kernels round (weights,
embedding, activations between hidden layers), FP32 everywhere else (the last hidden layer's
activations and the output layer)."""
import math

import numpy as np

OFF = {}
_sizes = [("emb", 64 * 16), ("W1", 128 * 32), ("b1", 128), ("W2", 128 * 128), ("b2", 128), ("W3", 128 * 128),
          ("b3", 128), ("w4", 128), ("b4", 4)]
_o = 0
for _n, _s in _sizes:
    OFF[_n] = (_o, _s)
    _o += _s
NPARAMS = _o
SHAPES = {"emb": (64, 16), "W1": (128, 32), "W2": (128, 128), "W3": (128, 128)}
LOSS_SCALE = 20.0


def split(flat, torch, requires_grad=False):
    out = {}
    for n, (o, s) in OFF.items():
        t = torch.tensor(np.asarray(flat[o:o + s], np.float32))
        if n in SHAPES:
            t = t.reshape(SHAPES[n])
        t.requires_grad_(requires_grad)
        out[n] = t
    return out


def bf(torch, t):
    """BF16-rounded value with an FP32 (straight-through) gradient, as the kernels' FP32 gradients
    see it; a plain cast would also round and accumulate the gradients in BF16."""
    return t + (t.to(torch.bfloat16).to(torch.float32) - t).detach()


def act(torch, z):
    """The kernels' activation, hard-swish: z * sat(z / 6 + 1/2) in FP32 (rounded to BF16 by the
    caller, as the kernels round it before the next layer)."""
    return z * torch.clamp(z * (1.0 / 6.0) + 0.5, 0.0, 1.0)


def row_outputs(torch, P, X, types):
    """y per row from features X (rows x 32, columns 16.. used as given; the embedding columns are
    rebuilt from P['emb'] so they carry gradients)."""
    x = torch.cat([bf(torch, P["emb"])[torch.as_tensor(types, dtype=torch.long)],
                   torch.as_tensor(X[:, 16:], dtype=torch.float32)], dim=1)
    h1 = bf(torch, act(torch, x @ bf(torch, P["W1"]).T + P["b1"]))
    h2 = bf(torch, act(torch, h1 @ bf(torch, P["W2"]).T + P["b2"]))
    h3 = act(torch, h2 @ bf(torch, P["W3"]).T + P["b3"])  # FP32: the output layer runs on the FMA pipe
    return h3 @ P["w4"] + P["b4"][0]


def pose_sums(torch, y, counts):
    idx = torch.as_tensor(np.repeat(np.arange(len(counts)), counts), dtype=torch.long)
    return torch.zeros(len(counts), dtype=torch.float32).index_add(0, idx, y)


def loss(torch, pred, labels):
    lab = torch.as_tensor(np.asarray(labels, np.float32))
    c = lambda e: LOSS_SCALE * torch.asinh(e / LOSS_SCALE)  # noqa: E731
    return ((c(pred) - c(lab)) ** 2).mean()
