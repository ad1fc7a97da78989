"""C-ABI library and host logic, without a GPU."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ddd_gb300.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ddd_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_python_binding(pkg):
    assert _declared() == sorted(pkg.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(pkg):
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    lib = ctypes.CDLL(pkg.LIB_PATH)
    for name in _declared():
        assert hasattr(lib, name), name
    lib.ddd_version.restype = ctypes.c_int
    assert lib.ddd_version() == 100


def test_fails_loudly_without_gpu(pkg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    L = pkg.library()
    assert L.ddd_create(0) is None
    assert len(L.ddd_last_error(None)) > 0
    with pytest.raises(pkg.DDDError):
        pkg.Context(0)


def test_material_constants_match_reference_formulas(pkg, fixtures):
    m = pkg.MaterialParameters(mu=1.0, nu=0.28)
    assert (m.μ4π, m.μ8π, m.μ4πν, m.νμ4πν) == fixtures.material_constants(1.0, 0.28)
    # sampleMaterialParameters.json stores the values the reference computes.
    assert m.μ4π == 0.07957747154594767 and m.μ8π == 0.039788735772973836
    assert abs(m.μ4πν - 0.11052426603603843) < 1e-17
    d = pkg.DislocationParameters(coreRad=90.78)
    assert d.coreRadSq == 90.78 * 90.78


def test_synthetic_loops_closed_and_sized(synth):
    p, b = synth.square_loops(200, 3, 20.0, 200.0, 20000.0, 0.5, 0.2)
    seg = np.roll(p, -1, axis=1) - p
    L = np.linalg.norm(seg, axis=2)
    assert np.allclose(L, L[:, :1], rtol=1e-12)  # 8 equal segments per loop
    assert np.all((L[:, 0] >= 20.0 - 1e-9) & (L[:, 0] <= 200.0 + 1e-9))
    assert np.abs(seg.sum(axis=1)).max() < 1e-9 * L.max()  # closed
    # Segments are perpendicular to b (shear loops: edge/screw mix is about n, but
    # every side lies in the slip plane or is an edge segment of the prism).
    assert np.all(np.abs(np.linalg.norm(b, axis=1) - 1) < 1e-15)


def test_synthetic_network_layout(synth):
    p, b = synth.square_loops(5, 1, 20.0, 200.0, 2000.0)
    coord, bvec, seg = synth.network_arrays(p, b)
    soa = synth.packed_soa(p, b)
    assert coord.flags.f_contiguous and seg.flags.f_contiguous
    for s in range(40):
        l, a, c = seg[s]
        assert np.array_equal(coord[:, a - 1], soa[0:3, s])
        assert np.array_equal(coord[:, c - 1], soa[3:6, s])
        assert np.array_equal(bvec[:, l - 1], soa[6:9, s])


def test_near_parallel_neighbours_present(synth):
    p, b = synth.square_loops(400, 2, 20.0, 200.0, 20000.0, 0.5, 0.05)
    n1 = p.reshape(-1, 3)
    t = (np.roll(p, -1, axis=1) - p).reshape(-1, 3)
    t /= np.linalg.norm(t, axis=1)[:, None]
    C = t @ t.T
    om = 1 - C * C
    iu = np.triu_indices(len(t), 1)
    tiny = om[iu][(om[iu] > 0) & (om[iu] <= 1.4901161193847656e-08)]
    assert len(tiny) > 0  # tilted copies give 0 < 1 - c^2 <= sqrt(eps)


def test_python_mirror_argument_checks(pkg):
    with pytest.raises(AssertionError):
        pkg.calc_σTilde_inplace(np.zeros((6, 3)), np.zeros((3, 4)), None, None, None)


def test_dislocation_parameters_assertions(pkg):
    """DislocationConstructor.jl:75-78: coreRad < minSegLen < maxSegLen unless
    all three are 0; minArea < maxArea unless both are 0."""
    d = pkg.DislocationParameters(coreRad=2.0)  # defaults 4 and 40: accepted
    assert (d.minSegLen, d.maxSegLen) == (4.0, 40.0)
    assert d.minArea == 16.0 / np.sqrt(2) and d.maxArea == 100 * d.minArea
    pkg.DislocationParameters(coreRad=0.0, minSegLen=0.0, maxSegLen=0.0, minArea=0.0, maxArea=0.0)
    for kw in (dict(coreRad=5.0, minSegLen=5.0), dict(coreRad=1.0, minSegLen=10.0, maxSegLen=9.0),
               dict(coreRad=1.0, minSegLen=2.0, maxSegLen=2.0), dict(coreRad=0.0, minSegLen=0.0, maxSegLen=1.0),
               dict(coreRad=1.0, minArea=5.0, maxArea=5.0), dict(coreRad=1.0, minArea=0.0, maxArea=-1.0)):
        with pytest.raises(AssertionError):
            pkg.DislocationParameters(**kw)


def test_product_iterator_points(pkg):
    """Iterators.product(xs, ys, zs) enumerates the first factor fastest; the
    mirror's ProductIterator gives calc_σTilde the points in that order, and
    calc_σTilde! rejects it as the reference's ndims assertion does."""
    xs, ys, zs = [0.0, 1.0, 2.0], [10.0, 20.0], [-5.0, 5.0, 7.0, 9.0]
    it = pkg.ProductIterator(xs, ys, zs)
    P = it.points()
    assert P.shape == (3, 24) and len(it) == 24
    want = [(x, y, z) for z in zs for y in ys for x in xs]  # Julia's order
    assert [tuple(P[:, j]) for j in range(24)] == want
    with pytest.raises(AssertionError):
        pkg.calc_σTilde_inplace(np.zeros((6, 24)), it, None, None, None)


# Julia struct of the shim -> C struct of the header.
JULIA_STRUCTS = {"DDDConsts": "ddd_consts", "DDDSelfParams": "ddd_self_params", "DDDMobParams": "ddd_mob_params",
                 "DDDCollision": "ddd_collision", "DDDUMesh": "ddd_u_mesh", "DDDSurOpts": "ddd_sur_opts",
                 "DDDSurReport": "ddd_sur_report"}
_C_TYPES = {"double": "f64", "int": "i32", "int32_t": "i32", "int64_t": "i64", "const double*": "ptr"}
_JL_TYPES = {"Float64": "f64", "Cint": "i32", "Int32": "i32", "Int64": "i64", "Ptr{Float64}": "ptr"}


def _c_struct_fields(text, name):
    m = re.search(r"typedef struct(?: \w+)? \{([^{}]*)\} " + name + ";", text)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        t = re.match(r"(const double\*|double|int64_t|int32_t|int)\s+(.*)", decl)
        assert t, decl
        for var in t.group(2).split(","):
            var = var.strip()
            a = re.match(r"(\w+)\[(\d+)\]$", var)
            fields.append((a.group(1), _C_TYPES[t.group(1)], int(a.group(2))) if a else
                          (var, _C_TYPES[t.group(1)], 1))
    return fields


def _jl_struct_fields(text, name):
    m = re.search(r"^struct " + name + r"\n(.*?)^end", text, re.S | re.M)
    assert m, name
    fields = []
    for line in m.group(1).strip().splitlines():
        var, typ = [x.strip() for x in line.split("::")]
        a = re.match(r"NTuple\{(\d+), (\w+)\}", typ)
        fields.append((var, _JL_TYPES[a.group(2)], int(a.group(1))) if a else (var, _JL_TYPES[typ], 1))
    return fields


def test_julia_shim_structs_match_header():
    """Every struct the Julia binding passes by reference has the header's
    fields, in order, with the same widths (a missing trailing field would let
    the library read past the caller's struct)."""
    jl = open(os.path.join(ROOT, "ddd.jl_gb300", "julia", "DDDGB300.jl")).read()
    c = open(HEADER).read()
    for jname, cname in JULIA_STRUCTS.items():
        assert _jl_struct_fields(jl, jname) == _c_struct_fields(c, cname), jname


def _ctypes_fields(cls):
    kinds = {ctypes.c_double: "f64", ctypes.c_int: "i32", ctypes.c_int32: "i32", ctypes.c_int64: "i64",
             ctypes.POINTER(ctypes.c_double): "ptr"}
    out = []
    for name, typ in cls._fields_:
        if issubclass(typ, ctypes.Array):
            out.append((name, kinds[typ._type_], typ._length_))
        else:
            out.append((name, kinds[typ], 1))
    return out


_ABI_STRUCTS = ("ddd_consts", "ddd_report", "ddd_self_params", "ddd_mob_params", "ddd_collision", "ddd_u_mesh",
                "ddd_batch_info_t", "ddd_sur_opts", "ddd_sur_report")


def test_python_structs_match_header(pkg, tmp_path):
    """Every ctypes struct of the Python mirror has the header's fields, in
    order, with the same widths, and the size the C compiler gives the
    header's struct (the ABI these pointers cross)."""
    c = open(HEADER).read()
    for cname in _ABI_STRUCTS:
        assert _ctypes_fields(getattr(pkg, cname)) == _c_struct_fields(c, cname), cname
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "ddd_gb300.h"\nint main(void) {\n' + "".join(
        '  printf("%%zu\\n", sizeof(%s));\n' % n for n in _ABI_STRUCTS) + "  return 0;\n}\n")
    exe = str(tmp_path / "sizes")
    r = subprocess.run([cc, "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", exe], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [ctypes.sizeof(getattr(pkg, n)) for n in _ABI_STRUCTS]


def test_quadrature_option_defaults(pkg):
    """The Python mirror's far-field options: the quadrature's own trust
    factors (QUAD_KAPPA for 3 points, QUAD2_KAPPA for 2), the 2-point switch
    at QUAD_KAPPA_TWO lengths for 3 points only, the network's checkpoint
    kappa otherwise; explicit values pass through."""
    import types
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))
    me = types.SimpleNamespace(kappa=20.0, nu=None)
    o = pkg.Surrogate._opts(me, k, None, 0.01, 1e-3, "f32c", "quad3")
    assert (o.kappa, o.kappa_two, o.far_mode, o.exact_mode) == (pkg.QUAD_KAPPA, pkg.QUAD_KAPPA_TWO, 3,
                                                                  pkg.MODES["f32c"])
    o = pkg.Surrogate._opts(me, k, None, 0.01, 1e-3, "fp64", "quad2")
    assert (o.kappa, o.kappa_two, o.far_mode) == (pkg.QUAD2_KAPPA, 0.0, 2)
    o = pkg.Surrogate._opts(me, k, None, 0.01, 1e-3, "fp64", "network")
    assert (o.kappa, o.kappa_two, o.far_mode) == (20.0, 0.0, 0)
    o = pkg.Surrogate._opts(me, k, 12.0, 0.0, 0.0, "fp64_fast", "quad3", 0.0)
    assert (o.kappa, o.kappa_two, o.audit_fraction) == (12.0, 0.0, 0.0)
