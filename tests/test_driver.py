"""mmh_recon, the reference's driver program (mmh/main.f90) on the library:
file names and formats as main.f90 builds them, its input checks, and on the
GPU its outputs against the same calls through the Python binding, and a
restart from its checkpoint against the uninterrupted run."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(os.path.dirname(HERE), "moving-mesh-reconstruction_gb300", "_build", "mmh_recon")


@pytest.fixture(scope="module")
def exe(mmh):
    mmh.lib()  # builds the library and the driver
    assert os.path.exists(EXE)
    return EXE


def run(exe, *args):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True)


def test_driver_file_names(exe):
    """main.f90:61, 122, 135-147, 166, 189-194, 208-213 with its defaults."""
    r = run(exe, "--ng", 512, "--niter", 300, "--restart", 150, "--print-names")
    assert r.returncode == 0, r.stderr
    names = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert names == {
        "input": "./0.000den0512_2.bin",
        "restart_u": "./u512/0.000restartu0150-_20512.bin",
        "restart_def": "./def512/0.000restartdef0150-_20512.bin",
        "checkpoint_u": "./u512/0.000restartu0300-_20512.bin",
        "checkpoint_def": "./def512/0.000restartdef0300-_20512.bin",
        "def": "./def512/0.000def_20512.bin",
        "psix": "./disp512/0.000psix_20512.bin",
        "psiy": "./disp512/0.000psiy_20512.bin",
        "psiz": "./disp512/0.000psiz_20512.bin",
        "recon": "./delta512/0.000recon_20512.bin",
    }


def test_driver_input_checks(exe, tmp_path):
    """A density whose mean is not 1 stops the program (main.f90:72-77); a
    missing or short file is an error.  Neither reaches the GPU."""
    n = 16
    wd = str(tmp_path) + "/"
    np.full(n ** 3, 1.1, dtype=np.float32).tofile(wd + "0.000den0016_2.bin")
    r = run(exe, "--ng", n, "--niter", 1, "--workdir", wd)
    assert r.returncode == 1 and "umean should be zero" in r.stdout
    r = run(exe, "--ng", 32, "--niter", 1, "--workdir", wd)
    assert r.returncode == 1 and "cannot read" in r.stderr
    assert run(exe, "--ng", n, "--bogus").returncode == 2


def _setup(tmp_path, rho, real8=False):
    wd = str(tmp_path) + "/"
    for d in ("u512", "def512", "delta512", "disp512"):
        os.makedirs(wd + d, exist_ok=True)
    n = rho.shape[0]
    rho.astype(np.float64 if real8 else np.float32).ravel(order="F").tofile(wd + f"0.000den{n:04d}_2.bin")
    return wd


def _load(path, n, real8=False, comps=1):
    a = np.fromfile(path, dtype=np.float64 if real8 else np.float32)
    assert a.size == comps * n ** 3
    return a.reshape((n, n, n) if comps == 1 else (n, n, n, comps), order="F")


@pytest.mark.gpu
def test_driver_matches_binding(exe, mmh, fields, tmp_path):
    n, niter = 32, 3
    rho = fields.lognormal_density(n, sigma=0.8, seed=77).astype(np.float32).astype(np.float64)
    wd = _setup(tmp_path, rho)
    r = run(exe, "--ng", n, "--niter", niter, "--workdir", wd, "--ps-dir", wd)
    assert r.returncode == 0, r.stderr + r.stdout
    assert r.stdout.count(" iter=") == niter
    u = np.zeros((5, n, n, n), order="F")
    u[0] = rho
    with mmh.Context(n, precision=mmh.MMH_FP64, schedule=mmh.MMH_SCHED_REF) as ctx:
        ctx.load(np.zeros((n, n, n), order="F"), u)
        ctx.iterate(niter)
        st = ctx.stats()
        d = np.zeros((n, n, n), order="F")
        uu = np.zeros((5, n, n, n), order="F")
        ctx.store(d, uu)
        grad = np.zeros((n, n, n, 3), order="F")
        delta = np.zeros((n, n, n), order="F")
        ctx.outputs(grad, delta)
        spectra = {"ps48bins_": ctx.power_spectrum(np.asfortranarray(rho - 1.0)),
                   "ps48bins_def_": ctx.power_spectrum(d)}
    # the Fisher script's inputs (calcfisherinfo.f90:26-27): "k P" per bin, k in rad/cell
    for stem, (k, p, _) in spectra.items():
        got = np.loadtxt(wd + f"{stem}{n}_2.txt")
        assert got.shape == (48, 2)
        np.testing.assert_allclose(got[:, 0], k * 2 * np.pi / n, rtol=1e-15)
        np.testing.assert_allclose(got[:, 1], p, rtol=1e-15)
    f32 = np.float32
    assert np.array_equal(_load(wd + f"def512/0.000def_2{n:04d}.bin", n), d.astype(f32))
    for a, ax in enumerate("xyz"):
        assert np.array_equal(_load(wd + f"disp512/0.000psi{ax}_2{n:04d}.bin", n), grad[..., a].astype(f32))
    assert np.array_equal(_load(wd + f"delta512/0.000recon_2{n:04d}.bin", n), delta.astype(f32))
    assert np.array_equal(_load(wd + f"u512/0.000restartu{niter:04d}-_2{n:04d}.bin", n), uu[0].astype(f32))
    # the last iteration's diagnostics (main.f90:97-105)
    last = r.stdout[r.stdout.rindex(" iter="):]
    printed = {k: float(last.split(k)[1].split()[0]) for k in ("defp sigma=", "def sigma=", "u sigma=")}
    assert printed["def sigma="] == pytest.approx(np.sqrt(np.mean(d ** 2)), rel=1e-6)
    assert printed["u sigma="] == pytest.approx(np.sqrt(np.mean((uu[0] - 1) ** 2)), rel=1e-6)
    assert printed["defp sigma="] == pytest.approx(st["defp_sigma"], rel=1e-6)
    assert st["rho_mean"] == pytest.approx(np.mean(uu[0]), rel=1e-12)
    assert st["rho_min"] == uu[0].min() and st["rho_max"] == uu[0].max()
    assert st["rho_negative"] == int((uu[0] < 0).sum())


@pytest.mark.gpu
def test_driver_restart_continues_the_run(exe, fields, tmp_path):
    """Checkpoint after 2 iterations, restart for the 3rd: the outputs are
    those of 3 uninterrupted iterations (8-byte files keep the state exact)."""
    n = 32
    rho = fields.lognormal_density(n, sigma=0.8, seed=78)
    straight = _setup(tmp_path / "a", rho, real8=True)
    split = _setup(tmp_path / "b", rho, real8=True)
    common = ["--ng", n, "--real8", "--schedule", "tol", "--tol", "1e-10"]
    assert run(exe, *common, "--niter", 3, "--workdir", straight).returncode == 0
    r = run(exe, *common, "--niter", 2, "--workdir", split, "--no-def", "--no-gradient", "--no-density")
    assert r.returncode == 0, r.stderr
    r = run(exe, *common, "--niter", 3, "--restart", 2, "--workdir", split)
    assert r.returncode == 0, r.stderr
    assert "RESTART!" in r.stdout and r.stdout.count(" iter=") == 1
    for name in (f"def512/0.000def_2{n:04d}.bin", f"delta512/0.000recon_2{n:04d}.bin",
                 f"disp512/0.000psiz_2{n:04d}.bin", f"u512/0.000restartu0003-_2{n:04d}.bin"):
        assert np.array_equal(_load(straight + name, n, True), _load(split + name, n, True)), name
