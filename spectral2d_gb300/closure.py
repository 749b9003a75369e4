"""Learned-closure LES workflow: data from the FP64 DNS, training, evaluation.

    python -m spectral2d_gb300.closure --out results.json --weights net.npz

1. Data: for each training seed, a decaying-turbulence DNS (N = 2048 by
   default, FP64, nu = 1e-4, dt from CFL 0.5 of the initial condition) spins
   up, then every ``every`` steps its state is sharp-filtered to the LES modes
   (|k| <= 64 for the 128^2 LES) and the subgrid flux
   Pi^ = T[N_dns(w)] - N_les(T w) is formed; (w, psi, Pi) on the LES
   collocation grid (192^2) become one training pair.
2. Training: Adam (lr 1e-3, batch 64) over the pairs of the training seeds,
   the last 10% held out as validation.
3. Evaluation on held-out seeds: the DNS and two 128^2 LES runs (FP32 by
   default; the DNS that makes the data stays FP64) started from the
   filtered DNS state -- one with the trained closure, one without (the
   fallback) -- advance with the same dt; the energy spectra E(k) of the LES
   runs are compared with the filtered DNS for k <= 40, together with the
   enstrophy, and the wall-clock per step of each solver is measured.

Everything runs on the GPU through ``libspectral2d_gb300.so``.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import solver as S


def _spectrum(h):
    k, Ek, tke, _, _ = h.compute_spectrum()
    return Ek, tke, h.enstrophy()


def generate(net, seeds, n_dns, n_les, nu, cfl, spinup, nsnap, every, log=print):
    """Fill the network's dataset with nsnap pairs per seed; returns the DNS
    dt of each seed and the seconds spent."""
    net.reserve(len(seeds) * nsnap)
    t0 = time.time()
    dts = {}
    with S.Spectral2D(n_les, nu=nu) as les:
        for s in seeds:
            with S.Spectral2D(n_dns, nu=nu) as dns:
                dns.set_turbulent_velocity(seed=s, spectrum="k4gauss", k0=10.0, tke=0.5)
                dt = dns.compute_time_step(cfl)
                dts[s] = dt
                dns.integrate_steps(spinup, dt)
                for _ in range(nsnap):
                    dns.integrate_steps(every, dt)
                    S.subgrid_flux(dns, les)
                    net.add_sample(les)
                dns.check_finite()
            log(f"seed {s}: {nsnap} pairs, dt {dt:.3e}, {time.time() - t0:.1f} s")
    return dts, time.time() - t0


def train(net, n, epochs, batch, lr, log=print):
    nval = max(batch, n // 10)
    ntr = n - nval
    hist = []
    t0 = time.time()
    for e in range(epochs):
        tr = net.train_epoch(0, ntr, batch, lr, seed=1000 + e)
        va = net.eval(ntr, nval)
        hist.append((tr, va))
        if e % 10 == 0 or e == epochs - 1:
            log(f"epoch {e}: train {tr:.4f} val {va:.4f} ({time.time() - t0:.1f} s)")
    return hist, time.time() - t0


def _rel_err(a, b, kmax):
    k = np.arange(1, kmax + 1)
    return np.abs(a[k] - b[k]) / np.abs(b[k])


def evaluate(net, seeds, n_dns, n_les, nu, cfl, steps, every, les_precision="fp32", log=print):
    """DNS vs LES with and without the closure on held-out seeds."""
    out = []
    for s in seeds:
        with S.Spectral2D(n_dns, nu=nu) as dns, S.Spectral2D(n_les, nu=nu) as filt, \
                S.Spectral2D(n_les, nu=nu, precision=les_precision) as les_c, \
                S.Spectral2D(n_les, nu=nu, precision=les_precision) as les_0:
            dns.set_turbulent_velocity(seed=s, spectrum="k4gauss", k0=10.0, tke=0.5)
            dt = dns.compute_time_step(cfl)
            S.filter_state(dns, les_c)
            S.filter_state(dns, les_0)
            S.les_set_closure(les_c, net)
            rec = {"seed": s, "dt": dt, "t": [], "err_closure": [], "err_none": [],
                   "enst_dns": [], "enst_closure": [], "enst_none": [], "tke_dns": [],
                   "tke_closure": [], "tke_none": []}
            t_dns = t_c = t_0 = 0.0
            for done in range(0, steps, every):
                n = min(every, steps - done)
                dns.synchronize()
                a = time.perf_counter()
                dns.integrate_steps(n, dt)
                dns.synchronize()
                b = time.perf_counter()
                S.les_integrate_steps(les_c, n, dt)
                les_c.synchronize()
                c = time.perf_counter()
                les_0.integrate_steps(n, dt)
                les_0.synchronize()
                d = time.perf_counter()
                t_dns += b - a
                t_c += c - b
                t_0 += d - c
                S.filter_state(dns, filt)
                Ef, tf, zf = _spectrum(filt)
                Ec, tc, zc = _spectrum(les_c)
                E0, t0_, z0 = _spectrum(les_0)
                rec["t"].append((done + n) * dt)
                rec["err_closure"].append(_rel_err(Ec, Ef, 40).tolist())
                rec["err_none"].append(_rel_err(E0, Ef, 40).tolist())
                for key, v in (("enst_dns", zf), ("enst_closure", zc), ("enst_none", z0),
                               ("tke_dns", tf), ("tke_closure", tc), ("tke_none", t0_)):
                    rec[key].append(v)
            les_c.check_finite()
            S.les_set_closure(les_c, None)
            rec["ms_per_step"] = {"dns": 1e3 * t_dns / steps, "les_closure": 1e3 * t_c / steps,
                                  "les_none": 1e3 * t_0 / steps}
            ec = np.array(rec["err_closure"])
            e0 = np.array(rec["err_none"])
            rec["summary"] = {
                "mean_rel_err_k_le_40_closure_final": float(ec[-1].mean()),
                "mean_rel_err_k_le_40_none_final": float(e0[-1].mean()),
                "mean_rel_err_k_le_40_closure_time_avg": float(ec.mean()),
                "mean_rel_err_k_le_40_none_time_avg": float(e0.mean()),
                "max_rel_err_k_le_40_closure_final": float(ec[-1].max()),
                "max_rel_err_k_le_40_none_final": float(e0[-1].max()),
                "speedup_vs_dns": t_dns / t_c,
            }
            log(f"seed {s}: {json.dumps(rec['summary'])}")
            out.append(rec)
    return out


def save_weights(net, path):
    np.savez_compressed(path, params=net.get_params(), scales=net.get_scales(), grid=net.grid)


def load_weights(net, path):
    d = np.load(path)
    net.set_params(d["params"])
    net.set_scales(d["scales"])


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-dns", type=int, default=2048)
    ap.add_argument("--n-les", type=int, default=128)
    ap.add_argument("--nu", type=float, default=1e-4)
    ap.add_argument("--cfl", type=float, default=0.5)
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--snaps", type=int, default=500)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--spinup", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-seeds", type=str, default="8,9")
    ap.add_argument("--eval-steps", type=int, default=20000)
    ap.add_argument("--eval-every", type=int, default=1000)
    ap.add_argument("--les-precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--weights", default=None)
    ap.add_argument("--load", default=None, help="skip data and training; use these weights")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    grid = 3 * a.n_les // 2
    res = {"config": vars(a)}
    with S.ClosureNet(grid, max_batch=a.batch, seed=0) as net:
        if a.load:
            load_weights(net, a.load)
        else:
            seeds = list(range(a.train_seeds))
            dts, tg = generate(net, seeds, a.n_dns, a.n_les, a.nu, a.cfl, a.spinup, a.snaps, a.every)
            rms = net.dataset_stats()
            net.set_scales(rms)
            hist, tt = train(net, net.dataset_size, a.epochs, a.batch, a.lr)
            res.update({"pairs": net.dataset_size, "data_seconds": tg, "train_seconds": tt,
                        "rms": rms.tolist(), "loss_history": hist})
            if a.weights:
                save_weights(net, a.weights)
        ev = [int(s) for s in a.eval_seeds.split(",") if s]
        res["eval"] = evaluate(net, ev, a.n_dns, a.n_les, a.nu, a.cfl, a.eval_steps, a.eval_every,
                               a.les_precision)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f)
    return res


if __name__ == "__main__":
    main()
