"""GPU tests of Analysis' skewness, checkpoints (bitwise resume) and restart
files (physical Omega, Psi, u, v + XDMF) against the oracle."""

import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S2D(built_lib):
    from spectral2d_gb300 import Spectral2D
    return Spectral2D


@pytest.mark.parametrize("n", [32, 128])
def test_skewness_vs_oracle(S2D, n):
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 40 + n, decay=0.05)
    with S2D(n, nu=0.01) as s:
        s.set_state(w)
        xs, ys = s.skewness()
        wd, pd = s.get_state()
    xo, yo = O.skewness(wd, pd, g)
    assert abs(xs - xo) <= 1e-12 * abs(xo) and abs(ys - yo) <= 1e-12 * abs(yo)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_checkpoint_resume_is_bitwise(S2D, tmp_path, precision):
    n, dt = 64, 1e-3
    path = str(tmp_path / "run.ckpt")
    with S2D(n, nu=2e-3, precision=precision) as a:
        a.set_turbulent_velocity(seed=9, spectrum="k4gauss", k0=6.0)
        a.integrate_steps(5, dt)
        a.checkpoint_write(path, nadv=5, time=5 * dt)
        a.integrate_steps(7, dt)
        wa, _ = a.get_state()
    with S2D(n, nu=2e-3, precision=precision) as b:
        nadv, t = b.checkpoint_read(path)
        assert nadv == 5 and t == 5 * dt
        b.integrate_steps(7, dt)
        wb, _ = b.get_state()
    assert np.array_equal(wa, wb)
    with S2D(32, nu=2e-3, precision=precision) as c:
        from spectral2d_gb300 import S2DError
        with pytest.raises(S2DError):
            c.checkpoint_read(path)


def test_restart_files_vs_oracle_and_reload(S2D, tmp_path):
    n = 48
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 3, decay=0.1)
    root = str(tmp_path / "REST")
    with S2D(n, nu=0.01) as s:
        s.set_state(w)
        wd, pd = s.get_state()
        binpath = s.write_restart(root, 1, nadv=123, time=0.5)
    M = g.nxG
    raw = open(binpath, "rb").read()
    assert raw[:8] == b"S2DREST1"
    hdr = np.frombuffer(raw[8:24], dtype=np.int32)
    assert tuple(hdr) == (n, n, M, M)
    assert np.frombuffer(raw[24:32], dtype=np.int64)[0] == 123
    assert np.frombuffer(raw[32:48], dtype=np.float64).tolist() == [0.5, 0.01]
    f = np.frombuffer(raw[64:], dtype=np.float64).reshape(4, M, M)
    u, v = O.compute_velocity(pd, g)
    for k, ref in enumerate((wd, pd, u, v)):
        phys = O.transform_c2r(ref, g)
        assert O.rel_l2(f[k], phys) < 1e-13
    xmf = open(root + "_00000001.xmf").read()
    assert 'Name="Omega"' in xmf and f'Seek="{64 + 3 * M * M * 8}"' in xmf
    with S2D(n, nu=0.01) as r:
        nadv, t = r.read_restart(binpath)
        w2, _ = r.get_state()
    assert (nadv, t) == (123, 0.5)
    assert O.rel_l2(w2, wd) < 1e-14
