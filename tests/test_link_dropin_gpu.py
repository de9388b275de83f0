"""Link-level drop-in on the GPU: a C++ program written against the reference's
declaration of ts::zquatev (zquatev.h:54), compiled with g++ without any header
of this project and linked against libzquatev_gb300.so in place of the
reference, solves the config-0 matrix (n2 = 512) and a small golden matrix.
Its output is compared with the compiled reference's (golden fixtures)."""
import os
import subprocess

import numpy as np
import pytest

from zquatev_gb300 import _lib, inputs, metrics

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-12


@pytest.fixture(scope="module")
def dropin_exe(gpu, tmp_path_factory):
    out = tmp_path_factory.mktemp("dropin") / "dropin_main"
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++11", os.path.join(HERE, "dropin_link", "main.cc"), "-o", str(out),
           "-L" + libdir, "-lzquatev_gb300", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


def run_exe(exe, d, tmp_path):
    ld2, n2 = d.shape
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    np.asfortranarray(d).ravel(order="F").tofile(fin)
    r = subprocess.run([exe, str(n2), str(ld2), str(fin), str(fout)], capture_output=True, text=True, timeout=300)
    raw = np.fromfile(fout, dtype=np.uint8)
    info = int(raw[:4].view(np.int32)[0])
    eig = raw[4:4 + 8 * n2].view(np.float64)
    out = raw[4 + 8 * n2:].view(np.complex128).reshape((ld2, n2), order="F")
    assert r.returncode == 0 and info == 0, (r.returncode, info, r.stderr)
    return out, eig


def test_cxx_caller_config0(dropin_exe, tmp_path):
    from tests.golden import make_golden

    z = np.load(os.path.join(HERE, "golden", "sketch_random_n256.npz"))
    n = int(z["n"])
    d = make_golden.sketched_input(str(z["kind"]), n, int(z["seed"]))
    d[:, n:] = 5.0 + 2.0j  # the right half is not read
    out, eig = run_exe(dropin_exe, d, tmp_path)
    assert np.all(eig[n:] == 7.25)  # eig[n..] untouched
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    hn = metrics.h_norm2(z["eig"])
    assert metrics.eig_error(eig[:n], z["eig"], hn) <= TOL
    assert metrics.residual(h, out, eig[:n]) <= TOL
    assert metrics.orthonormality(out) <= TOL
    assert metrics.structure_exact(out, n)
    s = metrics.sketch_matrix(2 * n, int(z["sketch_k"]), int(z["sketch_seed"]))
    assert metrics.sketch_distance(out, eig[:n], z["sketch"], z["eig"], s, 1e-5 * hn) < 1e-8


def test_cxx_caller_golden_n100(dropin_exe, tmp_path):
    z = np.load(os.path.join(HERE, "golden", "random_n100.npz"))
    left = z["left"]
    n = left.shape[1]
    d = np.zeros((2 * n, 2 * n), dtype=np.complex128, order="F")
    d[:, :n] = left
    out, eig = run_exe(dropin_exe, d, tmp_path)
    hn = metrics.h_norm2(z["eig"])
    assert metrics.eig_error(eig[:n], z["eig"], hn) <= TOL
    assert metrics.subspace_distance(out, eig[:n], z["out"], z["eig"], 1e-6 * hn) < 1e-8
    assert metrics.structure_exact(out, n)
