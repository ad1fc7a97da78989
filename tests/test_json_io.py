"""The reference's JSON formats: loadNetwork / saveJSON(network) and the
parameter loaders (src/IO/Input.jl, src/IO/Output.jl).

The reference's own IO test (test/ioTest.jl) is a round trip: a network saved
with saveJSON and read back with loadNetwork compares equal.  Here the same,
plus the on-disk layout JSON.jl gives the DislocationNetwork struct, and the
reference's sample parameter files (tests/golden/sample_params.json): the
material file stores Julia-computed derived constants, which the loader must
reproduce exactly.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

P = json.load(open(os.path.join(GOLDEN, "sample_params.json")))
FIELDS = ["numNode", "numSeg", "maxConnect", "label", "links", "connectivity", "linksConnect", "slipPlane", "extSeg",
          "segIdx", "bVec", "coord", "nodeVel", "nodeForce", "segForce"]


def test_material_parameters(pkg):
    d = P["materialParameters"]
    mat = pkg.json_io.loadMaterialParameters(d)
    for k in ("omνInv", "νomνInv", "μ4π", "μ8π", "μ4πν"):
        assert getattr(mat, k) == d[k], k
    assert mat.ν == 0.28 and mat.σPN == 0.0 and mat.crystalStruct == "DDD.BCC()"


def test_dislocation_parameters(pkg):
    d = P["dislocationParameters"]
    dln = pkg.json_io.loadDislocationParameters(d)
    assert dln.coreRadSq == d["coreRadSq"]
    assert dln.collisionDistSq == d["collisionDist"] * d["collisionDist"]
    assert dln.dragCoeffs == d["dragCoeffs"]
    assert (dln.minSegLen, dln.maxSegLen, dln.parGPU) == (d["minSegLen"], d["maxSegLen"], d["parGPU"])


def test_slip_system(pkg):
    d = P["slipSystem"]
    ss = pkg.json_io.loadSlipSystem(d)
    assert ss["slipPlane"].shape == (3, len(d["slipPlane"]))
    assert np.array_equal(ss["bVec"][:, 5], d["bVec"][5])


def _network(pkg, synth, seed=3):
    p, b = synth.square_loops(40, seed, 50.0, 200.0, 3000.0, 0.5, 0.05)
    coord, bvec, seg = synth.network_arrays(p, b)
    rng = np.random.default_rng(seed)
    net = pkg.DislocationNetwork(coord, bvec, seg, label=rng.integers(1, 6, coord.shape[1]),
                                 nodeVel=rng.normal(size=coord.shape), nodeForce=rng.normal(size=coord.shape),
                                 slipPlane=rng.normal(size=bvec.shape))
    net.segForce[...] = rng.normal(size=net.segForce.shape)
    net.linksConnect[...] = rng.integers(0, 4, net.linksConnect.shape)
    return net


def test_round_trip(pkg, synth, tmp_path):
    net = _network(pkg, synth)
    path = str(tmp_path / "network.json")
    pkg.saveJSON(path, net)
    back = pkg.loadNetwork(path)
    for name in ("coord", "bVec", "segIdx", "links", "connectivity", "label", "nodeVel", "nodeForce", "segForce",
                 "slipPlane", "linksConnect"):
        assert np.array_equal(getattr(back, name), getattr(net, name)), name
    assert (back.numNode, back.numSeg, back.maxConnect) == (net.numNode, net.numSeg, net.maxConnect)
    assert not back.extSeg.any()  # loadNetwork does not read extSeg


def test_layout(pkg, synth, tmp_path):
    """JSON.jl's layout of the struct: fields in declaration order, matrices as
    lists of columns, numNode / numSeg as one-element lists, labels as Int."""
    net = _network(pkg, synth)
    path = str(tmp_path / "network.json")
    pkg.saveJSON(path, net)
    d = json.load(open(path))
    assert list(d) == FIELDS
    assert d["numNode"] == [net.numNode] and d["maxConnect"] == 4
    assert d["coord"][7] == net.coord[:, 7].tolist() and len(d["coord"]) == net.coord.shape[1]
    assert len(d["segIdx"]) == 3 and d["segIdx"][1] == net.segIdx[:, 1].tolist()
    assert d["segForce"][5] == [net.segForce[:, 0, 5].tolist(), net.segForce[:, 1, 5].tolist()]
    assert all(isinstance(v, int) for v in d["label"])


def test_load_julia_written(pkg):
    """A file in the layout DDD.jl writes (the TopologyTest.jl triangle, with
    buffers of 4 links / 4 nodes), read as the reference's loader reads it."""
    d = {"numNode": [3], "numSeg": [3], "maxConnect": 2, "label": [1, 1, 3, 0],
         "links": [[1, 2], [1, 3], [2, 3], [0, 0]],
         "connectivity": [[2, 1, 1, 2, 1], [2, 1, 2, 3, 1], [2, 2, 2, 3, 2], [0, 0, 0, 0, 0]],
         "linksConnect": [[1, 1], [2, 1], [2, 2], [0, 0]], "slipPlane": [[1.0, 1.0, 1.0]] * 4,
         "extSeg": [False, False, True, False], "segIdx": [[1, 2, 3, 0], [1, 1, 2, 0], [2, 3, 3, 0]],
         "bVec": [[1.0, 1.0, 1.0]] * 3 + [[0.0, 0.0, 0.0]], "coord": [[0.0, 0.0, 0.0], [0.5, 0.0, 0.0],
                                                                      [0.0, 1.0, 0.0], [0.0, 0.0, 0.0]],
         "nodeVel": [[0.0, 0.0, 0.0], [-1.0, 1.0, 0.0], [1.0, -1.0, 0.0], [0.0, 0.0, 0.0]],
         "nodeForce": [[0.0, 0.0, 0.0]] * 4, "segForce": [[[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]] * 4}
    net = pkg.loadNetwork(d)
    assert net.links[:, :3].T.tolist() == [[1, 2], [1, 3], [2, 3]]
    assert net.coord.shape == (3, 4) and net.coord[0, 1] == 0.5
    assert net.connectivity[:, 1].tolist() == [2, 1, 2, 3, 1] and net.label.tolist() == [1, 1, 3, 0]
    assert net.segIdx[:, 1].tolist() == [1, 1, 2, 0] and (net.numNode, net.numSeg) == (3, 3)
    assert not net.extSeg.any()


@pytest.mark.gpu
def test_loaded_network_forces(pkg, fixtures, tmp_path):
    """A network read back from JSON gives the same seg-seg forces, bit for bit."""
    g = json.load(open(os.path.join(GOLDEN, "segseg_goldens.json")))
    c = g["cases"][0]
    fnet = fixtures.make_network(c["loops"], g["slipSystems"], c["range"], c["shift"])
    net = pkg.DislocationNetwork(fnet.coord, fnet.bVec, fnet.segIdx)
    dln = pkg.DislocationParameters(coreRad=g["params"]["coreRad"])
    mat = pkg.MaterialParameters(mu=g["params"]["mu"], nu=g["params"]["nu"])
    path = str(tmp_path / "net.json")
    pkg.saveJSON(path, net)
    back = pkg.loadNetwork(path)
    assert np.array_equal(pkg.calcSegSegForce(dln, mat, back), pkg.calcSegSegForce(dln, mat, net))

