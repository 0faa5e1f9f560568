"""libewpt from plain C99 (tests/c/abi_drive.c): the header compiles as C,
the argument checks hold without a device, and on the GPU a C caller gets
the same snapshot row as the Python binding for the same inputs."""
import os
import subprocess

import numpy as np
import pytest

import ewpt

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    import build_lib

    lib = build_lib.build()
    libdir = os.path.dirname(lib)
    out = str(tmp_path_factory.mktemp("c") / "abi_drive")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c", "abi_drive.c"), "-o", out,
                    "-L", libdir, "-lewpt", f"-Wl,-rpath,{libdir}", "-lm"], check=True)
    return out


def test_c_caller_host_checks(exe):
    r = subprocess.run([exe, "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "host ok" in r.stdout


@pytest.mark.gpu
def test_c_caller_matches_python_binding(exe):
    n, steps = 20, 3
    r = subprocess.run([exe, "gpu", str(n), str(steps)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    vals = np.array([float(v) for v in r.stdout.split()])
    row_c, eb_c = vals[:20], vals[20]
    p = ewpt.Params(N=n)  # the defaults of ewpt_params_default(n) (test_abi checks them)
    R, w = 2.0 / np.sqrt(p.lam), 1.0 / (np.sqrt(p.lam) * p.vev)
    bub = np.array([[4, 5, 6, 1, 0, 0, 0], [n / 2.0, n / 2.0, n / 3.0, 0, 1, 0, 0],
                    [n - 3.0, 7, n / 2.0, 0, 0, 0.6, 0.8]])
    with ewpt.Lattice(p) as lat:
        lat.init_bubbles(bub, "tanh", R, w)
        lat.step(steps)
        row = lat.diagnostics()
        B = lat.fields("B")
    np.testing.assert_array_equal(row_c, row)
    eb = 0.5 * (B ** 2).sum() * p.dx ** 3
    assert eb_c == pytest.approx(eb, rel=1e-12) and eb_c == pytest.approx(row[7], rel=1e-11)
