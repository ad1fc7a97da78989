"""Extract the reference's golden vectors for the seg-seg force and σ̃ path.

Reads DDD.jl's own test files as text (no Julia needed) and writes the
matrices they assert against into JSON fixtures beside this script:

  segseg_goldens.json   test/SegmentForcesTest.jl:281-443 — three networks
                        (coincident pentagons, shifted pentagons, prismatic +
                        shear hexagons), f1 = segForce[:, 1, :]', f2 = segForce[:, 2, :]'
  selfforce_goldens.json test/SegmentForcesTest.jl:220-267 — calcSelfForce on
                        two prismatic pentagons (the second shifted by 10),
                        f1 = selfForce[1]', f2 = selfForce[2]'
  mobility_goldens.json test/MobilityTest.jl:5-93 — BCC dlnMobility on a shear
                        hexagon and a prismatic pentagon after calcSegForce!
                        (zero FE fields, so no PK term): node forces and velocities
  collision_goldens.json test/TopologyTest.jl:5-92 — detectCollision on a
                        triangle and a 4-node loop under 17 skip lists (hinge
                        and twoLine results), and test/MiscTest.jl:82-150 —
                        minimumDistance on 9 segment pairs
  u_tilde_goldens.json  test/DislocationFEMTest.jl:270-1000 — calc_uTilde on a
                        3 × 5 × 7 cuboid mesh (1013 × 1987 × 2999) with a
                        prismatic and a shear octagon at its centre: ux, uy, uz at
                        the cantilever's displacement nodes, and the full
                        calc_uTilde! vector
  sample_params.json    test/testData/sampleDislocationParameters.json,
                        sampleMaterialParameters.json and BCC.json as parsed
                        data (the JSON loaders' inputs; the material file also
                        holds Julia-computed derived constants)
  sigma_goldens.json    test/DislocationFEMTest.jl:5-155 — one edge and one
                        screw segment, σ̃ at a 3×3 grid (columns 5 and 6 of the
                        golden are (yz, xz), the code's order is (xz, yz))

Run once in a checkout that has the reference mounted:
    python tests/golden/extract_goldens.py /path/to/DDD.jl
The fixtures are committed; nothing at test time reads the reference.
"""
import ast
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _matrices(text, name):
    """All `name = [ ... ]` (optionally `name = s * [ ... ]`) literal matrices, in order."""
    out = []
    pat = re.compile(r"\b" + re.escape(name) + r"\s*=\s*(?:([0-9.eE+-]+)\s*\*\s*)?\[")
    pos = 0
    while True:
        m = pat.search(text, pos)
        if not m:
            break
        scale = float(m.group(1)) if m.group(1) else 1.0
        end = text.index("]", m.end())
        body = text[m.end():end]
        rows = []
        for line in body.strip().splitlines():
            line = line.strip()
            if not line:
                continue
            rows.append([float(v) * scale for v in line.split()])
        out.append(rows)
        pos = end
    return out


def _julia_matrix(body):
    """Rows of a one-line Julia matrix literal body ("1 1 2; 2 3 3")."""
    return [[float(v) for v in row.split()] for row in body.split(";")]


def _safe_value(expr, env):
    """Evaluates the small vector expressions of MiscTest.jl's minimumDistance
    block (zeros(3), ones(3), scalars times them, [1, 0, 0], eps(Float64)^2 and
    names assigned before) by walking the parsed tree; anything else raises."""
    import numpy as np

    def ev(n):
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Name) and n.id in env:
            return env[n.id]
        if isinstance(n, ast.List):
            return np.array([ev(e) for e in n.elts], dtype=np.float64)
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, ast.USub):
            return -ev(n.operand)
        if isinstance(n, ast.BinOp) and type(n.op) in (ast.Add, ast.Sub, ast.Mult, ast.Pow):
            a, b = ev(n.left), ev(n.right)
            return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b, ast.Pow: a ** b}[type(n.op)]
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and len(n.args) == 1:
            if n.func.id in ("zeros", "ones"):
                k = int(ev(n.args[0]))
                return np.zeros(k) if n.func.id == "zeros" else np.ones(k)
            if n.func.id == "eps" and isinstance(n.args[0], ast.Name) and n.args[0].id == "Float64":
                return float(np.finfo(np.float64).eps)
        raise ValueError("unsupported expression: " + ast.dump(n))

    return ev(expr)


def _comma_vector(block, name):
    m = re.search(r"\b" + re.escape(name) + r"\s*=\s*\[([^\]]*)\]", block)
    return [float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]


def u_tilde_goldens(ref):
    """The "Calculate uTilde" testset of DislocationFEMTest.jl."""
    t = open(os.path.join(ref, "test", "DislocationFEMTest.jl")).read()
    blk = t[t.index('@testset "Calculate uTilde"'):]
    num = lambda name: float(re.search(r"\b" + name + r"\s*=\s*([0-9.eE+-]+)", blk).group(1))
    vec = lambda name: [float(v) for v in re.search(name + r"\s*=\s*Float64\[([^\]]*)\]", blk).group(1).split(";")]
    dims = {k: num(k) for k in ("dx", "dy", "dz")}
    cells = {k: int(num(k)) for k in ("mx", "my", "mz")}
    seg_len = (dims["dx"] + dims["dy"] + dims["dz"]) / 30
    loops = []
    for kind in ("loopPrism", "loopShear"):
        assert kind + "()" in blk
        loops.append({"type": "prism" if kind == "loopPrism" else "shear", "numSides": 8, "nodeSide": 1,
                      "numLoops": 1, "segLen": seg_len, "slipSystemIdx": 1, "label": [1] * 8})
    centre = [dims["dx"] / 2, dims["dy"] / 2, dims["dz"] / 2]
    json.dump({"mesh": dict(dims, **cells), "nu": num("ν"), "mu": 1.0,
               "slipSystems": {"slipPlane": [vec("slipPlane")], "bVec": [vec("bVec")]},
               "loops": loops, "range": [[c, c] for c in centre],
               "ux": _comma_vector(blk, "uxTest"), "uy": _comma_vector(blk, "uyTest"),
               "uz": _comma_vector(blk, "uzTest"), "uTildeFull": _comma_vector(blk, "uTildeTest"),
               "rtol": 5e-5},
              open(os.path.join(HERE, "u_tilde_goldens.json"), "w"), indent=1)


def collision_goldens(ref):
    """detectCollision cases of TopologyTest.jl's "Collision detection" testset
    and the minimumDistance cases of MiscTest.jl."""
    top = open(os.path.join(ref, "test", "TopologyTest.jl")).read()
    a = top.index('@testset "Collision detection"')
    block = top[a:top.index("@testset", a + 10)]
    dpar = json.load(open(os.path.join(ref, "test", "testData", "sampleDislocationParameters.json")))
    nets = []
    for part in block.split("network = DislocationNetwork(")[1:]:
        fields = {}
        for m in re.finditer(r"(\w+)\s*=\s*\w*\[([^\]]*)\]", part.split("makeConnect!")[0]):
            fields[m.group(1)] = _julia_matrix(m.group(2))
        cases, pending = [], []
        tok = re.compile(r"detectCollision\(\s*dlnParams,\s*network,\s*(skipSegs|\[[^\]]*\])\s*,?\s*\)"
                         r"|==\s*\((true|false),\s*:(\w+),([^)]*)\)")
        for m in tok.finditer(part):
            if m.group(1) is not None:
                pending.append([[int(x), int(y)] for x, y in re.findall(r"\((\d+),\s*(\d+)\)", m.group(1))])
            else:
                nums = [v.strip() for v in m.group(4).split(",") if v.strip()]
                exp = [m.group(2) == "true", m.group(3)] + [int(v) for v in nums[:6]] + [float(v) for v in nums[6:]]
                cases += [{"skip": sk, "expected": exp} for sk in pending]
                pending = []
        nets.append({"links": fields["links"], "bVec": fields["bVec"], "coord": fields["coord"],
                     "label": [r[0] for r in fields["label"]], "nodeVel": fields["nodeVel"], "cases": cases})

    misc = open(os.path.join(ref, "test", "MiscTest.jl")).read().splitlines()
    first = next(k for k, ln in enumerate(misc) if "minimumDistance(" in ln)
    while not misc[first - 1].strip().startswith("@test"):
        first -= 1
    env, mcases, inputs = {}, [], None
    names = ["x0", "x1", "y0", "y1", "vx0", "vx1", "vy0", "vy1"]
    for ln in misc[first:]:
        t = ln.strip()
        if t.startswith("end"):
            break
        if "minimumDistance(" in t:
            inputs = {k: env[k].tolist() for k in names}
        elif t.startswith("@test (distSq, dDistSqDt, L1, L2) =="):
            exp = ast.parse(t.split("==", 1)[1].strip(), mode="eval").body
            mcases.append({"inputs": inputs, "expected": [_safe_value(e, {}) for e in exp.elts]})
        elif "=" in t and not t.startswith("@"):
            tree = ast.parse(t.replace(".+", "+").replace("^", "**"), mode="exec").body[0]
            tg = tree.targets[0]
            vals = tree.value.elts if isinstance(tree.value, ast.Tuple) else [tree.value]
            tnames = [e.id for e in tg.elts] if isinstance(tg, ast.Tuple) else [tg.id]
            for nm, v in zip(tnames, vals):
                env[nm] = _safe_value(v, env)
    json.dump({"collisionDist": float(dpar["collisionDist"]), "networks": nets, "minimumDistance": mcases},
              open(os.path.join(HERE, "collision_goldens.json"), "w"), indent=1)


def main(ref):
    seg = open(os.path.join(ref, "test", "SegmentForcesTest.jl")).read()
    # The first f1/f2 pair (SegmentForcesTest.jl:244-267) holds the self-force
    # goldens; the seg-seg goldens are the next three.
    self_f1, self_f2 = _matrices(seg, "f1")[0], _matrices(seg, "f2")[0]
    f1s = _matrices(seg, "f1")[1:]
    f2s = _matrices(seg, "f2")[1:]
    assert len(f1s) == 3 and len(f2s) == 3, (len(f1s), len(f2s))
    cases = [
        {
            "name": "pentagons_coincident",
            "source": "test/SegmentForcesTest.jl:281-324",
            "loops": [{"type": "prism", "numSides": 5, "nodeSide": 1, "numLoops": 2, "segLen": 10.0,
                       "slipSystemIdx": 4, "label": [1, 2, 1, 2, 1]}],
            "shift": None,
        },
        {
            "name": "pentagons_shifted",
            "source": "test/SegmentForcesTest.jl:326-370",
            "loops": [{"type": "prism", "numSides": 5, "nodeSide": 1, "numLoops": 2, "segLen": 10.0,
                       "slipSystemIdx": 4, "label": [1, 2, 1, 2, 1]}],
            "shift": {"fromNode": 6, "by": [20.0, 20.0, 20.0]},
        },
        {
            "name": "hexagons_prism_shear",
            "source": "test/SegmentForcesTest.jl:382-443",
            "loops": [
                {"type": "prism", "numSides": 6, "nodeSide": 1, "numLoops": 1, "segLen": 10.0,
                 "slipSystemIdx": 1, "label": [1, 2, 1, 2, 1, 2]},
                {"type": "shear", "numSides": 6, "nodeSide": 1, "numLoops": 1, "segLen": 10.0,
                 "slipSystemIdx": 1, "label": [1, 2, 1, 2, 1, 2]},
            ],
            "shift": None,
        },
    ]
    for c, f1, f2 in zip(cases, f1s, f2s):
        c["range"] = [[-100.0, 100.0], [-100.0, 100.0], [-100.0, 100.0]]
        c["f1"] = f1
        c["f2"] = f2
    params = {
        "source": "test/testData/sampleDislocationParameters.json, sampleMaterialParameters.json",
        "coreRad": 90.78, "mu": 1.0, "nu": 0.28,
    }
    bcc = json.load(open(os.path.join(ref, "test", "testData", "BCC.json")))
    json.dump({"params": params, "slipSystems": {"slipPlane": bcc["slipPlane"], "bVec": bcc["bVec"]},
               "cases": cases}, open(os.path.join(HERE, "segseg_goldens.json"), "w"), indent=1)
    dpar = json.load(open(os.path.join(ref, "test", "testData", "sampleDislocationParameters.json")))
    self_case = {
        "name": "pentagons_shifted_10",
        "source": "test/SegmentForcesTest.jl:220-267",
        "loops": [{"type": "prism", "numSides": 5, "nodeSide": 1, "numLoops": 2, "segLen": 10.0,
                   "slipSystemIdx": 4, "label": [1, 2, 1, 2, 1]}],
        "shift": {"fromNode": 6, "by": [10.0, 10.0, 10.0]},
        "range": [[-100.0, 100.0], [-100.0, 100.0], [-100.0, 100.0]],
        "f1": self_f1, "f2": self_f2,
    }
    json.dump({"params": dict(params, coreEnergy=float(dpar["coreEnergy"])),
               "slipSystems": {"slipPlane": bcc["slipPlane"], "bVec": bcc["bVec"]}, "cases": [self_case]},
              open(os.path.join(HERE, "selfforce_goldens.json"), "w"), indent=1)

    mob = open(os.path.join(ref, "test", "MobilityTest.jl")).read()
    mvel, mforce = _matrices(mob, "testVel")[0], _matrices(mob, "testForce")[0]
    ipar = json.load(open(os.path.join(ref, "inputs", "simParams", "sampleDislocationParameters.json")))
    mpar = json.load(open(os.path.join(ref, "inputs", "simParams", "sampleMaterialParameters.json")))
    json.dump({
        "source": "test/MobilityTest.jl:5-93; parameters inputs/simParams/sample*Parameters.json",
        "params": {"coreRad": float(ipar["coreRad"]), "coreEnergy": float(ipar["coreEnergy"]),
                   "mu": float(mpar["μ"]), "nu": float(mpar["ν"]), "sigmaPN": float(mpar["σPN"]),
                   "drag": {k: float(v) for k, v in ipar["dragCoeffs"].items()}},
        "slipSystems": {"slipPlane": bcc["slipPlane"], "bVec": bcc["bVec"]},
        "loops": [
            {"type": "shear", "numSides": 6, "nodeSide": 1, "numLoops": 1, "segLen": 10.0, "slipSystemIdx": 4,
             "label": [1, 2, 1, 2, 1, 1]},
            {"type": "prism", "numSides": 5, "nodeSide": 1, "numLoops": 1, "segLen": 10.0, "slipSystemIdx": 4,
             "label": [1, 2, 1, 2, 1]},
        ],
        "range": [[-100.0, 100.0], [-100.0, 100.0], [-100.0, 100.0]],
        "maxConnect": 4,
        "nodeVel": mvel, "nodeForce": mforce,
    }, open(os.path.join(HERE, "mobility_goldens.json"), "w"), indent=1)

    fem = open(os.path.join(ref, "test", "DislocationFEMTest.jl")).read()
    sig = _matrices(fem, "test_σTilde")
    assert len(sig) == 2, len(sig)
    scases = [
        {"name": "edge_segment", "source": "test/DislocationFEMTest.jl:5-78", "b": [1.0, 0.0, 0.0],
         "golden": sig[0]},
        {"name": "screw_segment", "source": "test/DislocationFEMTest.jl:80-155", "b": [0.0, 0.0, 1.0],
         "golden": sig[1]},
    ]
    for c in scases:
        # Nodes at z = -300, 0, 300; one link (1 -> 2); a = 5|b|; μ = 1, ν = 0.28;
        # points on the 3×3 grid x, y ∈ {-300, 0, 300}, z = 0, ordered X[:] (x outer).
        c["coord"] = [[0.0, 0.0, -300.0], [0.0, 0.0, 0.0], [0.0, 0.0, 300.0]]
        c["links"] = [[1, 2]]
        c["coreRad"] = 5.0
        c["mu"] = 1.0
        c["nu"] = 0.28
        c["golden_columns"] = ["xx", "yy", "zz", "xy", "yz", "xz"]
    json.dump({"cases": scases}, open(os.path.join(HERE, "sigma_goldens.json"), "w"), indent=1)
    collision_goldens(ref)
    u_tilde_goldens(ref)
    td = os.path.join(ref, "test", "testData")
    json.dump({k: json.load(open(os.path.join(td, f))) for k, f in
               (("dislocationParameters", "sampleDislocationParameters.json"),
                ("materialParameters", "sampleMaterialParameters.json"), ("slipSystem", "BCC.json"))},
              open(os.path.join(HERE, "sample_params.json"), "w"), indent=1, ensure_ascii=False)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python extract_goldens.py <DDD.jl checkout>")
    main(sys.argv[1])
