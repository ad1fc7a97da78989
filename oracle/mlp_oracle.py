"""CPU oracle of the far-field surrogate (test infrastructure only).

A float64 NumPy restatement of the surrogate's features (csrc/surrogate.cuh)
and of the MLP's forward pass, loss and gradients (csrc/surrogate_mlp.cu),
rounding to BF16 at the same points as the GPU (inputs, weights, hidden
activations, output gradient, hidden-layer gradients fed to the GEMMs), so the
GPU's gradients can be checked against it.  GELU uses the exact tanh here; the
GPU uses the hardware tanh approximation (relative error ~2^-11).
"""
import numpy as np

FEAT, HIDDEN, OUT, USED_OUT = 16, 128, 16, 12
OFF = {}
_o = 0
for name, size in (("W1", HIDDEN * FEAT), ("b1", HIDDEN), ("W2", HIDDEN * HIDDEN), ("b2", HIDDEN),
                   ("W3", HIDDEN * HIDDEN), ("b3", HIDDEN), ("W4", OUT * HIDDEN), ("b4", OUT)):
    OFF[name] = (_o, size)
    _o += size
NUM_PARAMS = _o
SHAPES = {"W1": (HIDDEN, FEAT), "W2": (HIDDEN, HIDDEN), "W3": (HIDDEN, HIDDEN), "W4": (OUT, HIDDEN),
          "b1": (HIDDEN,), "b2": (HIDDEN,), "b3": (HIDDEN,), "b4": (OUT,)}


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(flat):
    return {k: np.asarray(flat[o:o + n], dtype=np.float64).reshape(SHAPES[k]) for k, (o, n) in OFF.items()}


def pack(d):
    flat = np.zeros(NUM_PARAMS)
    for k, (o, n) in OFF.items():
        flat[o:o + n] = d[k].ravel()
    return flat


def gelu(x):
    u = 0.7978845608028654 * (x + 0.044715 * x ** 3)
    return 0.5 * x * (1.0 + np.tanh(u))


def gelu_grad(x):
    u = 0.7978845608028654 * (x + 0.044715 * x ** 3)
    th = np.tanh(u)
    du = 0.7978845608028654 * (1.0 + 3 * 0.044715 * x * x)
    return 0.5 * (1 + th) + 0.5 * x * (1 - th * th) * du


def features(r, ti, tj, bi, bj, Li, Lj, mu4pi):
    """Features (16) and frame of one pair, as pair_features in csrc/surrogate.cuh."""
    r = np.asarray(r, np.float64)
    R = np.sqrt(r @ r)
    e3 = r / R
    a = ti @ e3
    e1 = ti - a * e3
    n1 = e1 @ e1
    if n1 < 1e-10:
        ax = 1.0 if abs(e3[0]) < 0.9 else 0.0
        ay = 1.0 - ax
        e1 = np.array([ay * e3[2], -ax * e3[2], ax * e3[1] - ay * e3[0]])
        n1 = e1 @ e1
    e1 = e1 / np.sqrt(n1)
    e2 = np.cross(e3, e1)
    f = np.zeros(FEAT)
    f[:13] = [ti @ e1, a, tj @ e1, tj @ e2, tj @ e3, bi @ e1, bi @ e2, bi @ e3, bj @ e1, bj @ e2, bj @ e3,
              10 * Li / R, 10 * Lj / R]
    return f, (e1, e2, e3, mu4pi * Li * Lj / (R * R))


def forward(p, X):
    """Activations of the GPU's forward pass (BF16 rounding at the GEMM inputs)."""
    W = {k: bf16(p[k]) if k.startswith("W") else p[k] for k in p}
    H0 = bf16(X)
    Z1 = H0 @ W["W1"].T + p["b1"]
    H1 = bf16(gelu(Z1))
    Z2 = H1 @ W["W2"].T + p["b2"]
    H2 = bf16(gelu(Z2))
    Z3 = H2 @ W["W3"].T + p["b3"]
    H3 = bf16(gelu(Z3))
    Y = H3 @ W["W4"].T + p["b4"]
    return dict(W=W, H0=H0, Z1=Z1, H1=H1, Z2=Z2, H2=H2, Z3=Z3, H3=H3, Y=Y)


def loss_and_grads(flat, X, T):
    """Mean-square loss over the 12 used outputs and the flat gradient."""
    p = unpack(flat)
    a = forward(p, X)
    B = X.shape[0]
    D = (a["Y"] - T)[:, :USED_OUT]
    loss = float((D * D).sum() / (12.0 * B))
    dYf = np.zeros((B, OUT))
    dYf[:, :USED_OUT] = 2.0 * D / (12.0 * B)
    dY = bf16(dYf)
    W = a["W"]
    g = {}
    g["W4"] = dY.T @ a["H3"]
    g["b4"] = dY.sum(0)
    dH = dY @ W["W4"]
    dZf = dH * gelu_grad(a["Z3"])
    dZ = bf16(dZf)
    g["W3"] = dZ.T @ a["H2"]
    g["b3"] = dZf.sum(0)
    dH = dZ @ W["W3"]
    dZf = dH * gelu_grad(a["Z2"])
    dZ = bf16(dZf)
    g["W2"] = dZ.T @ a["H1"]
    g["b2"] = dZf.sum(0)
    dH = dZ @ W["W2"]
    dZf = dH * gelu_grad(a["Z1"])
    dZ = bf16(dZf)
    g["W1"] = dZ.T @ a["H0"]
    g["b1"] = dZf.sum(0)
    return loss, pack(g)
