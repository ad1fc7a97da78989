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
  sigma_goldens.json    test/DislocationFEMTest.jl:5-155 — one edge and one
                        screw segment, σ̃ at a 3×3 grid (columns 5 and 6 of the
                        golden are (yz, xz), the code's order is (xz, yz))

Run once in a checkout that has the reference mounted:
    python tests/golden/extract_goldens.py /path/to/DDD.jl
The fixtures are committed; nothing at test time reads the reference.
"""
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
