"""CPU oracle of the warm-start MLP (test infrastructure): forward pass,
mean-squared loss and gradients in FP64 with the GPU's BF16 rounding of
layer inputs and weights (round to nearest even), for checking the GPU's
own training kernels.  Layout of the parameters as mc_ctx_surrogate_params."""
import numpy as np

NI, NH, NO, NT = 80, 128, 48, 41
OFF = {"W1": (0, (NH, NI)), "b1": (NH * NI, (NH,))}
OFF["W2"] = (OFF["b1"][0] + NH, (NH, NH))
OFF["b2"] = (OFF["W2"][0] + NH * NH, (NH,))
OFF["W3"] = (OFF["b2"][0] + NH, (NO, NH))
OFF["b3"] = (OFF["W3"][0] + NO * NH, (NO,))
NPARAM = OFF["b3"][0] + NO


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


def forward(p, x, rounding=True):
    P = unpack(p)
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    a1 = np.maximum(r(x) @ r(P["W1"]).T + P["b1"], 0.0)
    a2 = np.maximum(r(a1) @ r(P["W2"]).T + P["b2"], 0.0)
    y = r(a2) @ r(P["W3"]).T + P["b3"]
    return a1, a2, y


def loss_and_grads(p, x, t, rounding=True):
    P = unpack(p)
    bf16_ = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    m = x.shape[0]
    a1, a2, y = forward(p, x, rounding)
    d = np.zeros_like(y)
    d[:, :NT] = y[:, :NT] - t[:, :NT]
    loss = float((d ** 2).sum() / (m * NT))
    dy = 2.0 * d / (m * NT)
    g = {"W3": dy.T @ bf16_(a2), "b3": dy.sum(0)}
    dz2 = (dy @ bf16_(P["W3"])) * (a2 > 0)
    g["W2"], g["b2"] = dz2.T @ bf16_(a1), dz2.sum(0)
    dz1 = (dz2 @ bf16_(P["W2"])) * (a1 > 0)
    g["W1"], g["b1"] = dz1.T @ bf16_(x), dz1.sum(0)
    return loss, g, y
