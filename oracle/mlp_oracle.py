"""CPU oracle of the warm-start MLP (test infrastructure): forward pass,
mean-squared loss and gradients in FP64 with the GPU's BF16 rounding of
layer operands (round to nearest even), for checking the GPU's own training
kernels.  Four layers 80 -> 256 -> 256 -> 256 -> 48 with ReLU on the hidden
ones; layout of the parameters as mc_ctx_surrogate_params."""
import numpy as np

NI, NH, NO, NT = 80, 256, 48, 41
SIZES = (NI, NH, NH, NH, NO)
OFF = {}
_o = 0
for _l in range(4):
    OFF["W%d" % (_l + 1)] = (_o, (SIZES[_l + 1], SIZES[_l]))
    _o += SIZES[_l + 1] * SIZES[_l]
    OFF["b%d" % (_l + 1)] = (_o, (SIZES[_l + 1],))
    _o += SIZES[_l + 1]
NPARAM = _o


def unpack(p):
    return {k: p[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in OFF.items()}


def pack(d):
    p = np.zeros(NPARAM, dtype=np.float32)
    for k, (o, s) in OFF.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k], dtype=np.float32).reshape(-1)
    return p


def bf16(a):
    """float32 -> bfloat16 -> float32, round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _r(rounding):
    return bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))


def forward(p, x, rounding=True):
    """Activations of the three hidden layers and the output."""
    P = unpack(p)
    r = _r(rounding)
    acts = []
    h = np.asarray(x, dtype=np.float64)
    for l in range(1, 5):
        z = r(h) @ r(P["W%d" % l]).T + P["b%d" % l]
        h = np.maximum(z, 0.0) if l < 4 else z
        acts.append(h)
    return acts[:3], acts[3]


def loss_and_grads(p, x, t, rounding=True):
    """Loss over the first NT outputs, gradients of every parameter, output.
    Rounding as the GPU's kernels: the forward pass rounds both operands;
    the data gradient rounds the weights, the weight gradient the layer
    inputs."""
    P = unpack(p)
    r = _r(rounding)
    m = x.shape[0]
    hidden, y = forward(p, x, rounding)
    ins = [np.asarray(x, dtype=np.float64)] + hidden
    d = np.zeros_like(y)
    d[:, :NT] = y[:, :NT] - t[:, :NT]
    loss = float((d ** 2).sum() / (m * NT))
    dz = 2.0 * d / (m * NT)
    g = {}
    for l in range(4, 0, -1):
        g["W%d" % l] = dz.T @ r(ins[l - 1])
        g["b%d" % l] = dz.sum(0)
        if l > 1:
            dz = (dz @ r(P["W%d" % l])) * (ins[l - 1] > 0)
    return loss, g, y
