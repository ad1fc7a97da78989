"""The reference's JSON files for networks and parameters.

loadNetwork mirrors src/IO/Input.jl:277-344 and saveJSON writes a
DislocationNetwork as the reference's saveJSON does (src/IO/Output.jl:1-51,
JSON.jl's struct serialisation): an object with the struct's fields in
declaration order (numNode, numSeg, maxConnect, label, links, connectivity,
linksConnect, slipPlane, extSeg, segIdx, bVec, coord, nodeVel, nodeForce,
segForce), every matrix as the list of its columns (segIdx, links x 3, as its
three columns), nodeTypeDln labels as integers, numNode and numSeg as
one-element lists.  So a network saved here loads in DDD.jl and the other way
round.  The parameter loaders mirror Input.jl:52-64 (MaterialParameters),
221-236 (SlipSystem) and 244-268 (DislocationParameters).
"""
import json

import numpy as np


def loadJSON(path):
    """loadJSON (Input.jl:7-10): the file as a dictionary."""
    with open(path) as f:
        return json.load(f)


def _columns(rows, nrow, ncol, dtype):
    """A nrow x ncol Fortran-ordered array from a list of columns (the first
    len(rows) columns filled, the rest zero, as the reference's loader does)."""
    out = np.zeros((nrow, ncol), dtype=dtype, order="F")
    for i, col in enumerate(rows):
        out[:, i] = col
    return out


def loadNetwork(src):
    """loadNetwork(file or dict): a DislocationNetwork.  Arrays are sized as the
    reference sizes them: link arrays by len(links), node arrays by len(coord)
    (connectivity, nodeVel and nodeForce get len(links) columns, filled for the
    first len(coord)); extSeg is not read (all false), as in the reference."""
    from . import DislocationNetwork  # the package's network type

    d = loadJSON(src) if isinstance(src, str) else src
    nl, nc = len(d["links"]), len(d["coord"])
    maxc = int(d["maxConnect"])
    links = _columns(d["links"], 2, nl, np.int64)
    links_connect = _columns(d["linksConnect"], 2, nl, np.int64)
    seg_force = np.zeros((3, 2, nl), np.float64, order="F")
    for i, f in enumerate(d["segForce"][:nl]):
        seg_force[:, 0, i] = f[0]
        seg_force[:, 1, i] = f[1]
    slip = _columns(d["slipPlane"][:nc], 3, nl, np.float64)
    bvec = _columns(d["bVec"][:nc], 3, nl, np.float64)
    coord = _columns(d["coord"], 3, nc, np.float64)
    vel = _columns(d["nodeVel"][:nc], 3, nl, np.float64)
    force = _columns(d["nodeForce"][:nc], 3, nl, np.float64)
    conn = _columns(d["connectivity"][:nc], 2 * maxc + 1, nl, np.int64)
    seg_idx = np.zeros((nl, 3), np.int64, order="F")
    for k in range(3):
        seg_idx[:, k] = d["segIdx"][k]
    label = np.asarray(d["label"], np.int32)
    return DislocationNetwork(coord, bvec, seg_idx, numSeg=int(d["numSeg"][0]), extSeg=np.zeros(nl, np.uint8),
                              segForce=seg_force, links=links, connectivity=conn, numNode=int(d["numNode"][0]),
                              nodeForce=force, nodeVel=vel, maxConnect=maxc, label=label, slipPlane=slip,
                              linksConnect=links_connect)


def network_dict(network):
    """The network as JSON.jl serialises the DislocationNetwork struct."""
    n = network
    cols = lambda a: np.asarray(a).T.tolist()
    return {
        "numNode": [int(n.numNode)],
        "numSeg": [int(n.numSeg)],
        "maxConnect": int(n.maxConnect),
        "label": [int(v) for v in n.label],
        "links": cols(n.links),
        "connectivity": cols(n.connectivity),
        "linksConnect": cols(n.linksConnect),
        "slipPlane": cols(n.slipPlane),
        "extSeg": [bool(v) for v in n.extSeg],
        "segIdx": cols(n.segIdx),
        "bVec": cols(n.bVec),
        "coord": cols(n.coord),
        "nodeVel": cols(n.nodeVel),
        "nodeForce": cols(n.nodeForce),
        "segForce": [[n.segForce[:, 0, i].tolist(), n.segForce[:, 1, i].tolist()] for i in range(n.segForce.shape[2])],
    }


def saveJSON(path, *objs):
    """saveJSON (Output.jl:46-51): one object is written as itself, several as a
    list; DislocationNetwork objects as network_dict gives them."""
    from . import DislocationNetwork

    conv = [network_dict(o) if isinstance(o, DislocationNetwork) else o for o in objs]
    with open(path, "w") as f:
        json.dump(conv[0] if len(conv) == 1 else conv, f)


def loadMaterialParameters(d):
    """loadMaterialParameters (Input.jl:52-64)."""
    from . import MaterialParameters

    return MaterialParameters(crystalStruct=d["crystalStruct"], mu=float(d["μ"]), muMag=float(d["μMag"]),
                              nu=float(d["ν"]), sigmaPN=float(d["σPN"]))


def loadSlipSystem(d):
    """loadSlipSystem (Input.jl:221-236): crystal structure and 3 x n slip
    planes and Burgers vectors."""
    return {"crystalStruct": d["crystalStruct"], "slipPlane": np.asarray(d["slipPlane"], np.float64).T.copy(order="F"),
            "bVec": np.asarray(d["bVec"], np.float64).T.copy(order="F")}


def loadDislocationParameters(d):
    """loadDislocationParameters (Input.jl:244-268)."""
    from . import DislocationParameters

    keep = ("remesh", "collision", "separation", "virtualRemesh", "mobility")
    return DislocationParameters(coreRad=float(d["coreRad"]), dragCoeffs=d["dragCoeffs"],
                                 coreRadMag=float(d["coreRadMag"]), coreEnergy=float(d["coreEnergy"]),
                                 minSegLen=float(d["minSegLen"]), maxSegLen=float(d["maxSegLen"]),
                                 collisionDist=float(d["collisionDist"]), parCPU=bool(d["parCPU"]),
                                 parGPU=bool(d["parGPU"]), minArea=float(d["minArea"]), maxArea=float(d["maxArea"]),
                                 **{k: d[k] for k in keep})
