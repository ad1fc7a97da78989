"""The C ABI from a plain C host (tests/c_host/ddd_c_host.c): the header and
libddd_gb300.so are all a Julia ccall / cgo / JNI binding needs.

Without a GPU: the program compiles against include/ddd_gb300.h, links the
library, and ddd_create reports the missing device (exit 3, a message), with
no crash.  On the GPU: its all-pairs forces, idx-form forces and σ̃ are the
Python path's bit for bit (same library, same inputs), the banded form (the
partial-sum limit set from C) equals them to rounding, and an out-of-range
node number gives DDD_ERANGE with a message and leaves the context usable.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c_host", "ddd_c_host.c")


def _compile(pkg, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    libdir = os.path.dirname(pkg.LIB_PATH)
    exe = str(tmp_path / "ddd_c_host")
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir,
           "-lddd_gb300", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _write_input(path, k, net, x0, idx):
    with open(path, "wb") as f:
        np.array([net.coord.shape[1], net.numSeg, x0.shape[1], len(idx)], np.int64).tofile(f)
        np.array([k.aSq, k.mu4pi, k.mu8pi, k.mu4pinu, k.nuMu4pinu], np.float64).tofile(f)
        np.asfortranarray(net.coord, np.float64).ravel(order="F").tofile(f)
        np.asfortranarray(net.bVec[:, :net.numSeg], np.float64).ravel(order="F").tofile(f)
        np.asfortranarray(net.segIdx[:net.numSeg], np.int64).ravel(order="F").tofile(f)
        np.asfortranarray(x0, np.float64).ravel(order="F").tofile(f)
        np.asarray(idx, np.int64).tofile(f)


def _network(pkg, synth):
    p, b = synth.square_loops(90, 12, 20.0, 200.0, 2000.0, 0.5, 0.1)
    coord, bvec, seg = synth.network_arrays(p, b)
    return pkg.DislocationNetwork(coord, bvec, seg)


def test_c_host_without_gpu(pkg, synth, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the GPU test runs the program)")
    exe = _compile(pkg, tmp_path)
    net = _network(pkg, synth)
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))
    _write_input(str(tmp_path / "in.bin"), k, net, np.zeros((3, 4)), [1])
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert r.stderr.startswith("ddd_create: ") and len(r.stderr.strip()) > len("ddd_create:")


@pytest.mark.gpu
def test_c_host_matches_python_path(pkg, synth, tmp_path):
    exe = _compile(pkg, tmp_path)
    net = _network(pkg, synth)
    n = net.numSeg
    dln, mat = pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28)
    k = pkg.consts_of(dln, mat)
    x0 = synth.grid_points(8, 2000.0)
    idx = [1, 7, n, 7, n // 2]
    _write_input(str(tmp_path / "in.bin"), k, net, x0, idx)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, (r.stdout, r.stderr)
    fields = dict(kv.split("=") for kv in r.stdout.split())
    assert fields["rc_range"] == "-2" and int(fields["msg_len"]) > 0
    assert int(fields["pairs_general"]) + int(fields["pairs_parallel"]) == n * (n - 1) // 2
    out = np.fromfile(str(tmp_path / "out.bin"), np.float64)
    m = x0.shape[1]
    F, Fi, S, Fb = np.split(out, np.cumsum([6 * n, 6 * len(idx), 6 * m]))
    assert np.array_equal(F.reshape(3, 2, n, order="F"), pkg.calcSegSegForce(dln, mat, net))
    assert np.array_equal(Fi.reshape(3, 2, len(idx), order="F"), pkg.calcSegSegForce(dln, mat, net, idx))
    assert np.array_equal(S.reshape(6, m, order="F"), pkg.calc_σTilde(x0, dln, mat, net))
    assert np.linalg.norm(Fb - F) <= 1e-13 * np.linalg.norm(F)
