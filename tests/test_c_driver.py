"""A compiled C caller of the ABI (tests/mmh_main.c, the reference's driver
loop mmh/main.f90:83-179 with the drop-in calls) builds against include/mmh.h
and the library; on the GPU it gives bit for bit what the same calls give
through the Python binding."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(ROOT, "moving-mesh-reconstruction_gb300", "_build")


def _build(tmp_path):
    exe = str(tmp_path / "mmh_main")
    cmd = ["gcc", "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "mmh_main.c"), "-L", LIBDIR, "-lmmh_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_builds(mmh, tmp_path):
    mmh.lib()  # the library is built
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_c_driver_matches_python_binding(mmh, fields, tmp_path):
    n, niter = 32, 2
    exe = _build(tmp_path)
    rho = fields.lognormal_density(n, sigma=0.8, seed=4242, dtype=np.float32)
    rho.ravel(order="F").tofile(str(tmp_path / "den.bin"))
    r = subprocess.run([exe, str(n), str(niter), str(tmp_path / "den.bin"), str(tmp_path) + "/c_"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert len(r.stdout.strip().splitlines()) == niter

    def load(name, shape):
        return np.fromfile(str(tmp_path / ("c_" + name)), dtype=np.float32).reshape(shape, order="F")

    u = np.zeros((5, n, n, n), dtype=np.float32, order="F")
    u[0] = rho
    defpot = np.zeros((n, n, n), dtype=np.float32, order="F")
    defp = np.zeros_like(defpot, order="F")
    tmp = np.zeros_like(defpot, order="F")
    tmp2 = np.zeros((n + 2, n, n), dtype=np.float32, order="F")
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_REF) as ctx:
        for _ in range(niter):
            ctx.calcdefp(defp, tmp, tmp2, defpot, u)
            defpot[...] = defpot + defp
            ctx.relaxing(u, defpot, defp)
        grad = np.zeros((n, n, n, 3), dtype=np.float32, order="F")
        delta = np.zeros((n, n, n), dtype=np.float32, order="F")
        ctx.scalar2gradient(defpot, grad, (n, n, n))
        ctx.defp2delta(defpot, delta, (n, n, n))
    assert np.array_equal(load("def.bin", (n, n, n)), defpot)
    assert np.array_equal(load("grad.bin", (n, n, n, 3)), grad)
    assert np.array_equal(load("delta.bin", (n, n, n)), delta)
