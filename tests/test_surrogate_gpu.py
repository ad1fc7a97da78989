"""Learned far-field surrogate: features, exact targets, gradients and training on the GPU.

Gradients of one forward/backward pass on the GPU (tcgen05 GEMMs, BF16
operands, FP32 accumulation) are checked against the float64 CPU oracle
(oracle/mlp_oracle.py), which rounds to BF16 at the same points; the remaining
difference is FP32 accumulation order and the GPU's hardware tanh (~2^-11), so
each parameter tensor must agree to 2e-2 in relative norm and the loss to 1e-3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(synth, loops=200, seed=5, cube=20000.0):
    p, b = synth.square_loops(loops, seed, 20.0, 200.0, cube, 0.5, 0.05)
    return p, b, synth.packed_soa(p, b)


def _far_pairs(soa, P, seed, rmin):
    rng = np.random.default_rng(seed)
    n = soa.shape[1]
    m = 0.5 * (soa[0:3] + soa[3:6])
    out = []
    while len(out) < P:
        i, j = rng.integers(0, n, 2)
        if i != j and np.linalg.norm(m[:, j] - m[:, i]) > rmin:
            out.append((i, j))
    return np.ascontiguousarray(np.array(out, dtype=np.int32).T)


def _k(pkg):
    return pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))


def test_features_and_exact_targets(pkg, synth, oracle):
    torch = pytest.importorskip("torch")
    from oracle import mlp_oracle as M
    p, b, soa = _net(synth)
    pairs = _far_pairs(soa, 256, 1, 2000.0)
    ctx = pkg.get_context()
    k = _k(pkg)
    dsoa = torch.from_numpy(soa).cuda()
    dpairs = torch.from_numpy(pairs).cuda()
    X = torch.zeros((256, 16), dtype=torch.float16, device="cuda")
    Bp = torch.zeros((256, 16), dtype=torch.float32, device="cuda")
    T = torch.zeros((256, 16), dtype=torch.float32, device="cuda")
    F = torch.zeros((256, 12), dtype=torch.float64, device="cuda")
    sur = pkg.Surrogate(ctx, seed=0)
    sur.make_data(k, dsoa.data_ptr(), soa.shape[1], dpairs.data_ptr(), 256, X.data_ptr(), Bp.data_ptr(),
                  T.data_ptr(), F.data_ptr())
    Xh, Bh, Th, Fh = X.float().cpu().numpy(), Bp.cpu().numpy(), T.cpu().numpy(), F.cpu().numpy()
    k5 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / 0.72, 0.28 / (4 * np.pi) / 0.72])
    for q in range(0, 256, 16):
        i, j = pairs[:, q]
        a1, a2, ab = soa[0:3, i], soa[3:6, i], soa[6:9, i]
        c1, c2, cb = soa[0:3, j], soa[3:6, j], soa[6:9, j]
        ref = oracle.pair(k5, ab, a1, a2, cb, c1, c2).ravel()
        # Far pairs: the formula cancels strongly, so two correct FP64 evaluations
        # agree to ~1e-6 of the largest component (measured against a long-double
        # evaluation of the same pairs).
        assert np.allclose(Fh[q], ref, rtol=0, atol=1e-5 * np.abs(ref).max())
        li, lj = np.linalg.norm(a2 - a1), np.linalg.norm(c2 - c1)
        f, bp, (e1, e2, e3, scale) = M.features(0.5 * (c1 + c2) - 0.5 * (a1 + a2), (a2 - a1) / li, (c2 - c1) / lj,
                                                ab, cb, li, lj, k5[1])
        assert np.allclose(Xh[q, :8], M.f16(f), atol=1e-3)
        assert np.allclose(Xh[q, :8] + Xh[q, 8:], f, rtol=1e-5, atol=1e-6)  # hi + lo
        assert np.allclose(Bh[q, :9], bp, rtol=1e-5, atol=1e-6) and np.all(Bh[q, 9:] == 0)
        E = np.stack([e1, e2, e3])
        for node in range(4):
            back = scale * (Th[q, 3 * node:3 * node + 3] @ E)
            assert np.allclose(back, ref[3 * node:3 * node + 3], rtol=1e-5, atol=1e-6 * np.abs(ref).max())


def _random_rows(rng, B):
    """Layer-1 rows, Burgers-vector products and targets of B random samples."""
    from oracle import mlp_oracle as M
    Xf = np.zeros((B, 8), np.float32)
    Xf[:, :7] = rng.uniform(-1, 1, (B, 7))
    bl, br = rng.uniform(-1, 1, (B, 3)), rng.uniform(-1, 1, (B, 3))
    Bpf = np.zeros((B, 16), np.float32)
    Bpf[:, :9] = (bl[:, :, None] * br[:, None, :]).reshape(B, 9)
    Tf = rng.normal(size=(B, 16)).astype(np.float32)
    Tf[:, 12:] = 0
    return M.split(Xf), Bpf, Tf


def test_gradients_match_cpu_oracle(pkg):
    torch = pytest.importorskip("torch")
    from oracle import mlp_oracle as M
    B = 256
    rng = np.random.default_rng(2)
    X16, Bpf, Tf = _random_rows(rng, B)
    sur = pkg.Surrogate(pkg.get_context(), seed=3)
    flat = sur.params()
    flat[M.OFF["b1"][0]:M.OFF["b1"][0] + 128] = rng.normal(0, 0.1, 128)  # non-zero biases too
    o4 = M.OFF["b4"][0]
    flat[o4:o4 + 108] = rng.normal(0, 0.1, 108)
    sur.set_params(flat)
    X = torch.from_numpy(X16.astype(np.float16)).cuda()
    Bp, T = torch.from_numpy(Bpf).cuda(), torch.from_numpy(Tf).cuda()
    loss, g = sur.grads(X.data_ptr(), Bp.data_ptr(), T.data_ptr(), B)
    ref_loss, ref_g = M.loss_and_grads(flat.astype(np.float64), X16, Bpf, Tf.astype(np.float64))
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss
    for name, (o, n) in M.OFF.items():
        a, r = g[o:o + n].astype(np.float64), ref_g[o:o + n]
        if name == "W4" or name == "b4":
            a, r = a.reshape(M.SHAPES[name])[:108], r.reshape(M.SHAPES[name])[:108]
        assert np.linalg.norm(a - r) <= 2e-2 * np.linalg.norm(r) + 1e-12, name


def test_training_reduces_loss_and_forward_matches(pkg, synth):
    torch = pytest.importorskip("torch")
    from oracle import mlp_oracle as M
    p, b, soa = _net(synth, loops=400, seed=8)
    P = 32768
    pairs = _far_pairs(soa, P, 4, 2000.0)
    ctx = pkg.get_context()
    sur = pkg.Surrogate(ctx, seed=1)
    X = torch.zeros((P, 16), dtype=torch.float16, device="cuda")
    Bp = torch.zeros((P, 16), dtype=torch.float32, device="cuda")
    T = torch.zeros((P, 16), dtype=torch.float32, device="cuda")
    dsoa, dpairs = torch.from_numpy(soa).cuda(), torch.from_numpy(pairs).cuda()  # kept alive across the call
    sur.make_data(_k(pkg), dsoa.data_ptr(), soa.shape[1], dpairs.data_ptr(), P, X.data_ptr(), Bp.data_ptr(),
                  T.data_ptr())
    assert torch.isfinite(X.float()).all() and torch.isfinite(T).all() and torch.isfinite(Bp).all()
    # Per-output normalisation, as Surrogate.fit trains.
    sig = torch.ones(16, device="cuda")
    sig[:12] = T[:, :12].std(0)
    Tn = (T / sig).contiguous()
    hist = sur.train(X.data_ptr(), Bp.data_ptr(), Tn.data_ptr(), P, 1024, 8, lr=2e-3)
    assert np.all(np.isfinite(hist)) and hist[-1] < 0.2 * hist[0]
    O = torch.zeros((P, 16), dtype=torch.float32, device="cuda")
    sur.forward(X.data_ptr(), Bp.data_ptr(), P, O.data_ptr())
    a = M.forward(M.unpack(sur.params().astype(np.float64)), X[:512].float().cpu().numpy(), Bp[:512].cpu().numpy())
    o = O[:512].cpu().numpy()
    assert np.all(o[:, 12:] == 0)
    assert np.abs(o[:, :12] - a["out"]).max() <= 2e-2 * np.abs(a["out"]).max()
