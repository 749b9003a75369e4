"""The main program's argument handling, on CPU: bad options and invalid
grids are rejected before any GPU work (exit codes 2 and 1)."""

import subprocess

import pytest


@pytest.fixture(scope="module")
def driver(built_lib):
    from spectral2d_gb300.build import DRIVER
    return DRIVER


def _run(driver, *args):
    return subprocess.run([driver, *map(str, args)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                          text=True, timeout=60)


def test_unknown_option_prints_usage(driver):
    p = _run(driver, "--bogus")
    assert p.returncode == 2 and "spectral2d_run" in p.stdout


def test_missing_value_and_bad_periods(driver):
    assert _run(driver, "--nx").returncode == 2
    assert _run(driver, "--print-period", 0).returncode == 2
    assert _run(driver, "--ic", "vortex").returncode == 2


@pytest.mark.parametrize("nx", [60, 4])
def test_invalid_grid_is_rejected_by_create(driver, tmp_path, nx):
    p = _run(driver, "--nx", nx, "--ny", nx, "--out", tmp_path)
    assert p.returncode == 1 and "s2d_create" in p.stdout and "multiple of 8" in p.stdout
    assert not (tmp_path / "EULERIAN.DAT").exists()


def test_nx_alone_sets_both_sizes(driver, tmp_path):
    """--nx without --ny gives a square grid: the rejection of nx = 60 is the
    grid's own (not a size mismatch), and a differing --ny is a mismatch."""
    p = _run(driver, "--nx", 60, "--out", tmp_path)
    assert p.returncode == 1 and "multiple of 8" in p.stdout
    p = _run(driver, "--nx", 16, "--ny", 32, "--out", tmp_path)
    assert p.returncode == 1 and "nx must equal ny" in p.stdout
