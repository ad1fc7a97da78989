"""Seeded synthetic dislocation networks for the parity tests and the benchmark.

A network is a set of closed square loops of 8 segments (numSides = 4,
nodeSide = 2 in the reference's DislocationLoop terms: src/Type/
DislocationConstructor.jl:196-298), each on a slip system drawn uniformly from
the 12 BCC {110}<111> systems (data/slipSystems/BCC.json), unit Burgers
vector, side 2L with L uniform in [Lmin, Lmax], centre uniform in a cube.
Shear loops turn about the slip-plane normal, prismatic loops about b.  A
fraction of loops is a copy of the previous loop shifted 2-10 b along its
slip-plane normal (exactly parallel neighbours); half of those copies are also
tilted by 1e-5 rad, so 0 < 1 - c^2 <= sqrt(eps) pairs are present too.

The node layout follows the reference's loop builder: node 1 at the origin,
sides added in turn, the closing link 8 -> 1 lying on side 1.
"""
import numpy as np

# BCC {110}<111> slip systems in the order of data/slipSystems/BCC.json.
BCC_SLIP_PLANES = np.array([[1, 1, 0], [1, 1, 0], [-1, 1, 0], [-1, 1, 0], [1, 0, 1], [1, 0, 1], [-1, 0, 1],
                            [-1, 0, 1], [0, 1, 1], [0, 1, 1], [0, -1, 1], [0, -1, 1]], dtype=np.float64)
BCC_BURGERS = np.array([[-1, 1, 1], [1, -1, 1], [1, 1, 1], [1, 1, -1], [1, 1, -1], [-1, 1, 1], [1, 1, 1], [1, 1, 1],
                        [1, -1, 1], [1, 1, -1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)

MU, NU, CORE_RAD = 1.0, 0.28, 1.0


def _unit(v):
    return v / np.sqrt((v * v).sum(axis=-1, keepdims=True))


def _rotate(v, axis, ang):
    """Rodrigues rotation of the rows of v about unit axis rows by ang."""
    c, s = np.cos(ang)[:, None], np.sin(ang)[:, None]
    return v * c + np.cross(axis, v) * s + axis * (axis * v).sum(-1, keepdims=True) * (1 - c)


def square_loops(num_loops, seed, lmin, lmax, cube, shear_fraction=1.0, parallel_fraction=0.0,
                 slip_subset=None):
    """Node coordinates (num_loops, 8, 3) and Burgers vectors (num_loops, 3)."""
    rng = np.random.default_rng(seed)
    systems = np.arange(12) if slip_subset is None else np.asarray(slip_subset)
    sidx = systems[rng.integers(0, len(systems), num_loops)]
    n = _unit(BCC_SLIP_PLANES[sidx])
    b = _unit(BCC_BURGERS[sidx])
    shear = rng.random(num_loops) < shear_fraction
    L = rng.uniform(lmin, lmax, num_loops)
    centre = rng.uniform(0.0, cube, (num_loops, 3))
    e1 = _unit(np.cross(n, b))  # edge direction (n × b)/|n × b|
    axis = np.where(shear[:, None], n, b)
    d = [e1, np.cross(axis, e1), -e1, -np.cross(axis, e1)]  # sides rotated by 0, 90, 180, 270 degrees
    Lv = L[:, None]
    p = np.zeros((num_loops, 8, 3))
    steps = [d[0], d[1], d[1], d[2], d[2], d[3], d[3]]  # node q+1 = node q + L * steps[q]
    for q in range(7):
        p[:, q + 1] = p[:, q] + Lv * steps[q]
    p -= p.mean(axis=1, keepdims=True)
    # Near-parallel neighbours: loop k becomes loop k-1 shifted along n (half of them tilted).
    if parallel_fraction > 0:
        pick = np.nonzero(rng.random(num_loops) < parallel_fraction)[0]
        pick = pick[pick > 0]
        shift = rng.uniform(2.0, 10.0, len(pick))
        tilt = rng.random(len(pick)) < 0.5
        for m, k in enumerate(pick):
            src = k - 1
            n[k], b[k], shear[k], L[k] = n[src], b[src], shear[src], L[src]
            off = p[src].copy()
            if tilt[m]:
                off = _rotate(off, np.repeat(_unit(np.cross(n[src], e1[src]))[None], 8, 0), np.full(8, 1e-5))
            p[k] = off
            centre[k] = centre[src] + shift[m] * n[src]
    p += centre[:, None, :]
    return p, b


def network_arrays(p, b):
    """Julia-layout arrays: coord (3×nodes), bVec (3×links), segIdx (links×3, 1-based)."""
    nl = p.shape[0]
    coord = np.asfortranarray(p.reshape(nl * 8, 3).T)
    bvec = np.asfortranarray(np.repeat(b, 8, axis=0).T)
    base = (np.arange(nl) * 8)[:, None]
    n1 = base + np.arange(8)[None, :] + 1
    n2 = base + (np.arange(8)[None, :] + 1) % 8 + 1
    links = np.arange(nl * 8) + 1
    seg = np.asfortranarray(np.stack([links, n1.ravel(), n2.ravel()], axis=1).astype(np.int64))
    return coord, bvec, seg


def packed_soa(p, b):
    """Device-form packed SoA (9 × N): n1 xyz, n2 xyz, b xyz per segment."""
    nl = p.shape[0]
    n1 = p.reshape(nl * 8, 3)
    n2 = np.roll(p, -1, axis=1).reshape(nl * 8, 3)
    bb = np.repeat(b, 8, axis=0)
    return np.ascontiguousarray(np.concatenate([n1.T, n2.T, bb.T], axis=0))


def grid_points(n, cube):
    """n^3 points at cell centres of a uniform grid over [0, cube]^3, x slowest (3 × n^3)."""
    c = (np.arange(n) + 0.5) * (cube / n)
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    return np.asfortranarray(np.stack([X.ravel(), Y.ravel(), Z.ravel()]))


# The workloads (segment count = 8 × loops).
CONFIGS = {
    # 64 shear loops, 512 segments, L ~ U(50, 200), 2000^3 cube, σ̃ on a 16^3 grid.
    "cpu512": dict(num_loops=64, lmin=50.0, lmax=200.0, cube=2000.0, shear_fraction=1.0, parallel_fraction=0.0,
                   grid=16),
    # 4096 shear + prismatic loops, 32,768 segments, L ~ U(20, 200), 20,000^3 cube,
    # 5% near-parallel neighbours, σ̃ on a 128^3 grid.
    "gpu32k": dict(num_loops=4096, lmin=20.0, lmax=200.0, cube=20000.0, shear_fraction=0.5, parallel_fraction=0.05,
                   grid=128),
    # The same generator at 65,536 segments (the headline pair-throughput workload).
    "gpu65k": dict(num_loops=8192, lmin=20.0, lmax=200.0, cube=20000.0, shear_fraction=0.5, parallel_fraction=0.05,
                   grid=128),
    # Precision form, 131,072 segments.
    "prec131k": dict(num_loops=16384, lmin=20.0, lmax=200.0, cube=20000.0, shear_fraction=0.5,
                     parallel_fraction=0.05, grid=128),
}


def make(config, seed=0, num_loops=None):
    """(p, b, cfg) for a named workload; num_loops overrides the size (same generator)."""
    cfg = dict(CONFIGS[config])
    if num_loops is not None:
        cfg["num_loops"] = int(num_loops)
    p, b = square_loops(cfg["num_loops"], seed, cfg["lmin"], cfg["lmax"], cfg["cube"], cfg["shear_fraction"],
                        cfg["parallel_fraction"])
    return p, b, cfg


def batch_networks(num_networks=256, seed=0, nmin=64, nmax=8192):
    """Independent networks for the batched form: segment counts log-uniform in
    [nmin, nmax] (rounded to whole 8-segment loops), each with its own seed, its
    own cube edge uniform in [2000, 20000] b and a random subset of the 12 slip
    systems; same loop generator otherwise.  Returns a list of (p, b)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(num_networks):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        loops = max(1, n // 8)
        cube = rng.uniform(2000.0, 20000.0)
        subset = np.sort(rng.choice(12, rng.integers(1, 13), replace=False))
        p, b = square_loops(loops, int(rng.integers(1 << 31)), 20.0, 200.0, cube, 0.5, 0.05, slip_subset=subset)
        out.append((p, b))
    return out
