"""CPU oracle of the far-field surrogate (test infrastructure only).

A float64 NumPy restatement of the surrogate's features and Burgers-vector
contraction (csrc/surrogate.cuh) and of the MLP's forward pass, loss and
gradients (csrc/surrogate_mlp.cu), rounding at the same points as the GPU: the
forward pass in FP16 (inputs, weights, hidden activations), the backward pass in
BF16 (the coefficient gradient, hidden-layer gradients, and BF16 copies of the
weights and activations fed to the backward GEMMs), so the GPU's gradients can
be checked against it.  GELU is the exact function here; the GPU evaluates it
on FP16 pairs with the hardware tanh approximation (a few FP16 ulps).

Model: the network maps the 8 geometric features of a pair (layer 1 takes each
as two FP16 numbers, hi = f16(f) and lo = f16(f - hi), against the weights
[W1 | W1], so its product is (hi + lo) W1^T) to 112 outputs Y, of which 108 are
the coefficients C[ac][o] = Y[12 ac + o] of the bilinear form
    out[o] = sum_ac Bp[ac] C[ac][o],   Bp[3 a + c] = (b_i.e_a)(b_j.e_c),
giving the 12 scaled node forces.
"""
import numpy as np

GEO, FEAT_IN, HIDDEN, OUT, USED_OUT, BPROD = 8, 16, 128, 112, 12, 9
COEF = BPROD * USED_OUT
OFF = {}
_o = 0
for name, size in (("W1", HIDDEN * GEO), ("b1", HIDDEN), ("W2", HIDDEN * HIDDEN), ("b2", HIDDEN),
                   ("W3", HIDDEN * HIDDEN), ("b3", HIDDEN), ("W4", OUT * HIDDEN), ("b4", OUT)):
    OFF[name] = (_o, size)
    _o += size
NUM_PARAMS = _o
SHAPES = {"W1": (HIDDEN, GEO), "W2": (HIDDEN, HIDDEN), "W3": (HIDDEN, HIDDEN), "W4": (OUT, HIDDEN),
          "b1": (HIDDEN,), "b2": (HIDDEN,), "b3": (HIDDEN,), "b4": (OUT,)}


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def f16(a):
    """Round to the nearest FP16 (ties to even), returned as float64."""
    return np.asarray(a, dtype=np.float32).astype(np.float16).astype(np.float64)


def split(f):
    """Layer-1 operand rows (..., 16) of geometric features f (..., 8): hi = f16(f)
    and lo = f16(f - hi), the difference taken in float32 (exact), as
    split_features in csrc/surrogate.cuh."""
    f32 = np.asarray(f, dtype=np.float32)
    hi = f16(f32)
    lo = f16(f32 - hi.astype(np.float32))
    return np.concatenate([hi, lo], axis=-1)


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
    """Geometric features (8), Burgers-vector products (9) and frame of one pair,
    as pair_features in csrc/surrogate.cuh."""
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
    f = np.zeros(GEO)
    f[:7] = [ti @ e1, a, tj @ e1, tj @ e2, tj @ e3, 10 * Li / R, 10 * Lj / R]
    E = np.stack([e1, e2, e3])
    bp = np.outer(E @ bi, E @ bj).ravel()
    return f, bp, (e1, e2, e3, mu4pi * Li * Lj / (R * R))


def contract(Y, Bp):
    """out[:, o] = sum_ac Bp[:, ac] Y[:, 12 ac + o] (Y already includes b4)."""
    C = Y[:, :COEF].reshape(-1, BPROD, USED_OUT)
    return np.einsum("pa,pao->po", Bp[:, :BPROD], C)


def forward(p, X, Bp=None):
    """Activations of the GPU's forward pass (FP16 rounding at the GEMM inputs);
    X holds layer-1 operand rows (B x 16, hi and lo parts, see split).  With Bp
    (B x 9 or wider), also the contracted outputs `out`."""
    W = {k: f16(p[k]) for k in p if k.startswith("W")}
    X = f16(X)
    H0 = X[:, :GEO] + X[:, GEO:]
    Z1 = H0 @ W["W1"].T + p["b1"]
    H1 = f16(gelu(Z1))
    Z2 = H1 @ W["W2"].T + p["b2"]
    H2 = f16(gelu(Z2))
    Z3 = H2 @ W["W3"].T + p["b3"]
    H3 = f16(gelu(Z3))
    Y = H3 @ W["W4"].T + p["b4"]
    a = dict(X=X, H0=H0, Z1=Z1, H1=H1, Z2=Z2, H2=H2, Z3=Z3, H3=H3, Y=Y)
    if Bp is not None:
        a["out"] = contract(Y, np.asarray(Bp, np.float64))
    return a


def loss_and_grads(flat, X, Bp, T):
    """Mean-square loss over the 12 contracted outputs and the flat gradient."""
    p = unpack(flat)
    Bp = np.asarray(Bp, np.float64)[:, :BPROD]
    a = forward(p, X, Bp)
    B = X.shape[0]
    D = a["out"] - np.asarray(T, np.float64)[:, :USED_OUT]
    loss = float((D * D).sum() / (12.0 * B))
    g_out = 2.0 * D / (12.0 * B)
    dYf = np.zeros((B, OUT))
    dYf[:, :COEF] = (Bp[:, :, None] * g_out[:, None, :]).reshape(B, COEF)
    dY = bf16(dYf)
    Wb = {k: bf16(p[k]) for k in p if k.startswith("W")}  # BF16 copies of the FP32 master weights
    X = a["X"]
    g = {}
    g["W4"] = dY.T @ bf16(a["H3"])
    g["b4"] = dYf.sum(0)
    dH = dY @ Wb["W4"]
    dZf = dH * gelu_grad(a["Z3"])
    dZ = bf16(dZf)
    g["W3"] = dZ.T @ bf16(a["H2"])
    g["b3"] = dZf.sum(0)
    dH = dZ @ Wb["W3"]
    dZf = dH * gelu_grad(a["Z2"])
    dZ = bf16(dZf)
    g["W2"] = dZ.T @ bf16(a["H1"])
    g["b2"] = dZf.sum(0)
    dH = dZ @ Wb["W2"]
    dZf = dH * gelu_grad(a["Z1"])
    dZ = bf16(dZf)
    g["W1"] = dZ.T @ (bf16(X[:, :GEO]) + bf16(X[:, GEO:]))
    g["b1"] = dZf.sum(0)
    return loss, pack(g)
