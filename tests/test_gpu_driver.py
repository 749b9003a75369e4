"""GPU tests of the main program ``spectral2d_run`` (src/Spectral2D.F90):
the print / write / stat cadences with the reference's one-step look-ahead,
the output formats, the DESIRED_END_TIME dt adjustment, and that its state
is the library's state after the same steps."""

import os
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(built_lib):
    from spectral2d_gb300.build import DRIVER
    assert os.path.exists(DRIVER), "spectral2d_run was not built"
    return DRIVER


def run(driver, out, *args):
    os.makedirs(out, exist_ok=True)
    p = subprocess.run([driver, "--out", str(out), *map(str, args)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert p.returncode == 0, p.stdout
    return p.stdout


def test_cadence_formats_and_state(driver, tmp_path):
    from spectral2d_gb300 import Spectral2D
    n, nu, dt, steps = 64, 2e-3, 1e-3, 25
    ck = tmp_path / "end.ckpt"
    log = run(driver, tmp_path, "--nx", n, "--ny", n, "--nu", nu, "--dt", dt, "--steps", steps,
              "--ic", "k4gauss", "--k0", 6.0, "--tke", 0.5, "--seed", 4, "--print-period", 10,
              "--stat-period", 10, "--write-period", 20, "--checkpoint", ck)
    # prints at 10, 20 and the last step; analysis at 0, 10, 20, 25; restarts at 0, 20, 25
    printed = [int(m) for m in re.findall(r"Simulation step number: (\d{8}); Simulation time:", log)]
    assert printed == [10, 20, 25]
    line = re.search(r"Simulation step number: 00000025; Simulation time: (.{15}); Max W: (.{15}); "
                     r"Min W: (.{15}); Max Psi: (.{15}); Min Psi: (.{15})$", log, re.M)
    assert line and float(line.group(1)) == pytest.approx(25 * dt, rel=1e-7)
    eul = open(tmp_path / "EULERIAN.DAT").read().splitlines()
    assert eul[0] == "# NADV          TIME            TKE             EPS             EnstDiss        xSkew           ySkew"
    rows = eul[1:]
    assert [r[:12] for r in rows] == ["  0000000000", "  0000000010", "  0000000020", "  0000000025"]
    assert all(len(r) == 12 + 6 * 16 for r in rows)
    for nadv in (0, 10, 20, 25):
        spec = open(tmp_path / f"SPECTRUM_{nadv:08d}.DAT").read().splitlines()
        assert spec[0].startswith("# k")
        assert spec[1][:6] == "000000" and spec[2][:6] == "000001"
    for num in range(3):
        assert os.path.exists(tmp_path / f"REST_{num:08d}.bin")
        assert os.path.exists(tmp_path / f"REST_{num:08d}.xmf")
    assert not os.path.exists(tmp_path / "REST_00000003.bin")

    # the same run through the library
    with Spectral2D(n, nu=nu) as s:
        s.set_turbulent_velocity(seed=4, spectrum="k4gauss", k0=6.0, tke=0.5)
        s.integrate_steps(steps, dt)
        wa, _ = s.get_state()
        _, Ek, tke, eps, enst = s.compute_spectrum()
        xs, ys = s.skewness()
        mm = s.minmax_abs()
    with Spectral2D(n, nu=nu) as r:
        nadv, t = r.checkpoint_read(str(ck))
        wb, _ = r.get_state()
    assert nadv == steps and t == pytest.approx(steps * dt, rel=1e-12)
    assert np.array_equal(wa, wb)
    last = [float(x) for x in rows[-1][12:].split()]
    assert np.allclose(last, [steps * dt, tke, eps, enst, xs, ys], rtol=1e-7, atol=0)
    assert [float(line.group(k)) for k in range(2, 6)] == pytest.approx(list(mm), rel=1e-7)
    spec = np.loadtxt(tmp_path / "SPECTRUM_00000025.DAT")
    assert np.allclose(spec[:, 1], Ek, rtol=1e-7, atol=1e-300)


def test_desired_end_time_lands_on_t_end(driver, tmp_path):
    from spectral2d_gb300 import Spectral2D
    n, nu, dt, t_end = 32, 0.01, 3e-3, 0.01   # 3 full steps + one of 1e-3
    ck = tmp_path / "end.ckpt"
    log = run(driver, tmp_path, "--nx", n, "--ny", n, "--nu", nu, "--dt", dt, "--end-time", t_end,
              "--ic", "tg", "--print-period", 1000, "--stat-period", 1000, "--write-period", 1000,
              "--checkpoint", ck)
    assert re.findall(r"Simulation step number: (\d{8})", log) == ["00000004"]
    t = 0.0
    for _ in range(3):   # the driver's time accumulation
        t = t + dt
    with Spectral2D(n, nu=nu) as s:
        s.set_taylor_green()
        s.integrate_steps(3, dt)
        s.integrate_one_step(t_end - t)
        wa, _ = s.get_state()
    with Spectral2D(n, nu=nu) as r:
        nadv, t = r.checkpoint_read(str(ck))
        wb, _ = r.get_state()
    assert nadv == 4 and t == pytest.approx(t_end, abs=1e-15)
    assert np.array_equal(wa, wb)
