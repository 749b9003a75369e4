"""Kolmogorov-forced turbulence: the FP64 and FP32 forms side by side.

    python -m spectral2d_gb300.kolmogorov --n 4096 --steps 10000 --out kolmo.json

The vorticity equation gains the source F = amp cos(k_f y) and the linear drag
-alpha w (terms added to dW, src/Spectral.F90:479).  Both forms start from the
same seeded state -- a k^4 exp(-2 (k/k0)^2) spectrum of small energy on top of
which the forcing builds the Kolmogorov shear -- and advance with one fixed dt:
CFL 0.5 of the larger of the initial velocity and the laminar Kolmogorov
velocity amp / (k_f (alpha + nu k_f^2)).  At every report point the FP32
form's energy spectrum E(k), its enstrophy and its vorticity are compared with
FP64's; the device time per step of each form is measured with CUDA events.
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import solver as S


def fixed_dt(h, n, nu, alpha, amp, kf, cfl):
    """One dt for the whole run (see the module docstring)."""
    dt_ic = h.compute_time_step(cfl)
    u_lam = amp / (kf * (alpha + nu * kf * kf)) if kf > 0 else 0.0
    m = 3 * n // 2
    dx = 2.0 * math.pi / m
    dt_lam = cfl / (2.0 * u_lam / dx) if u_lam > 0 else math.inf
    return min(dt_ic, dt_lam)


def compare(h64, h32, kmax):
    """FP32 vs FP64: max relative E(k) error for 1 <= k <= kmax, relative
    enstrophy error, relative L2 of the vorticity."""
    _, e64, tke64, _, _ = h64.compute_spectrum()
    _, e32, tke32, _, _ = h32.compute_spectrum()
    kk = slice(1, kmax + 1)
    rel = np.abs(e32[kk] - e64[kk]) / np.maximum(e64[kk], 1e-300)
    z64, z32 = h64.enstrophy(), h32.enstrophy()
    w64, _ = h64.get_state()
    w32, _ = h32.get_state()
    l2 = float(np.linalg.norm(w32 - w64) / np.linalg.norm(w64))
    return {"Ek_max_rel_err": float(rel.max()), "Ek_mean_rel_err": float(rel.mean()),
            "tke_rel_err": abs(tke32 - tke64) / tke64, "enstrophy_rel_err": abs(z32 - z64) / z64,
            "w_rel_l2": l2, "tke": tke64, "enstrophy": z64}


def run(n=4096, nu=1e-5, alpha=0.1, amp=4.0, kf=4, steps=10000, every=1000, cfl=0.5, seed=0,
        tke0=1e-3, k0=10.0, kmax=40, timing_steps=20, log=print):
    out = {"config": {"n": n, "padded": 3 * n // 2, "nu": nu, "alpha": alpha, "forcing": f"{amp} cos({kf} y)",
                      "steps": steps, "every": every, "cfl": cfl, "seed": seed, "ic_tke": tke0, "k0": k0,
                      "kmax_compare": kmax}}
    kw = dict(nu=nu, alpha=alpha, forcing_amp=amp, forcing_k=kf)
    with S.Spectral2D(n, precision="fp64", **kw) as h64, S.Spectral2D(n, precision="fp32", **kw) as h32:
        h64.set_turbulent_velocity(seed=seed, spectrum="k4gauss", k0=k0, tke=tke0)
        w0, _ = h64.get_state()
        h32.set_state(w0)
        dt = fixed_dt(h64, n, nu, alpha, amp, kf, cfl)
        out["dt"] = dt
        # device time per step of each form (the state advances; both forms
        # advance by the same number of steps, so they stay comparable)
        for name, h in (("fp64", h64), ("fp32", h32)):
            h.integrate_steps(3, dt)
            ms = h.time_steps(timing_steps, dt) / timing_steps
            out[name] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms,
                         "mpt_steps_per_s": n * n / 1e3 / ms}
            log(f"{name}: {ms:.3f} ms/step")
        done = 3 + timing_steps
        out["reports"] = []
        t0 = time.time()
        while done < steps:
            k = min(every, steps - done)
            h64.integrate_steps(k, dt)
            h32.integrate_steps(k, dt)
            done += k
            h64.check_finite()
            h32.check_finite()
            rep = {"step": done, "time": done * dt, **compare(h64, h32, kmax)}
            out["reports"].append(rep)
            log(f"step {done}: E(k) max rel err {rep['Ek_max_rel_err']:.3e}, enstrophy rel err "
                f"{rep['enstrophy_rel_err']:.3e}, w rel L2 {rep['w_rel_l2']:.3e} ({time.time() - t0:.0f} s)")
        out["wall_s"] = time.time() - t0
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--nu", type=float, default=1e-5)
    ap.add_argument("--alpha", type=float, default=0.1)
    ap.add_argument("--amp", type=float, default=4.0)
    ap.add_argument("--kf", type=int, default=4)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--every", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    res = run(n=a.n, nu=a.nu, alpha=a.alpha, amp=a.amp, kf=a.kf, steps=a.steps, every=a.every, seed=a.seed)
    txt = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt)
    print(txt)


if __name__ == "__main__":
    main()
