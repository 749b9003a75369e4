"""GPU test of the Kolmogorov-flow workflow (FP64 and FP32 forms side by
side) on a small grid."""

import pytest

pytestmark = pytest.mark.gpu


def test_fp32_tracks_fp64(built_lib):
    from spectral2d_gb300 import kolmogorov
    res = kolmogorov.run(n=128, nu=1e-3, steps=400, every=200, tke0=0.05, kmax=40, timing_steps=5,
                         log=lambda *a: None)
    assert res["fp64"]["ms_per_step"] > 0 and res["fp32"]["ms_per_step"] > 0
    last = res["reports"][-1]
    assert last["step"] == 400
    assert last["w_rel_l2"] < 1e-4 and last["Ek_max_rel_err"] < 1e-3
    assert last["enstrophy_rel_err"] < 1e-4
