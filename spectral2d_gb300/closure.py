"""Learned-closure LES workflow: data from the FP64 DNS, training, evaluation.

    python -m spectral2d_gb300.closure --out results.json --weights net.npz

1. Data: for each training seed (0-7), a decaying-turbulence DNS (N = 2048
   by default, FP64, nu = 1e-4, dt from CFL 0.5 of the initial condition);
   every ``every`` steps (40 by default, 500 snapshots: the whole 20000-step
   evaluation window) its state is sharp-filtered to the LES modes
   (|k| <= 64 for the 128^2 LES) and the subgrid flux
   Pi^ = T[N_dns(w)] - N_les(T w) is formed; (w, psi, Pi) on the LES
   collocation grid (192^2) become one training pair.
2. Training: Adam (lr 1e-3 on a cosine down to 5e-5, batch 64, 150 epochs)
   over the pairs, the last 10% held out as validation.  The band k_min
   below which the closure term is not applied is chosen on validation seed
   10 among --bands.
3. Evaluation on held-out seeds 8, 9: the DNS and 128^2 LES runs (FP32 by
   default; the DNS that makes the data stays FP64) started from the
   filtered DNS state -- with the trained closure and without (the
   fallback), at the DNS's dt and at multiples of it (--dt-factors) -- are
   compared every 1000 DNS steps: E(k) of the LES against the filtered DNS
   for k <= 40, the enstrophy, and the wall-clock of each solver over the
   same simulated time.

Everything runs on the GPU through ``libspectral2d_gb300.so``.
"""

from __future__ import annotations

import argparse
import json
import math
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


def train(net, n, epochs, batch, lr, lr_min_frac=0.05, log=print):
    """Adam over the first 90% of the pairs (the rest validates), the
    learning rate following a cosine from lr down to lr * lr_min_frac."""
    nval = max(batch, n // 10)
    ntr = n - nval
    hist = []
    t0 = time.time()
    for e in range(epochs):
        f = lr_min_frac + (1.0 - lr_min_frac) * 0.5 * (1.0 + math.cos(math.pi * e / max(1, epochs - 1)))
        tr = net.train_epoch(0, ntr, batch, lr * f, seed=1000 + e)
        va = net.eval(ntr, nval)
        hist.append((tr, va))
        if e % 10 == 0 or e == epochs - 1:
            log(f"epoch {e}: train {tr:.4f} val {va:.4f} lr {lr * f:.2e} ({time.time() - t0:.1f} s)")
    return hist, time.time() - t0


KMAX = 40   # spectra are compared for 1 <= k <= KMAX


def _rel_err(a, b):
    return np.abs(a - b) / np.abs(b)


def evaluate(net, seeds, n_dns, n_les, nu, cfl, steps, every, bands=(0.0,), les_precision="fp32",
             dt_factors=(1,), log=print):
    """The FP64 DNS against 128^2 LES runs started from its filtered state:
    one without closure (the fallback) and one with the closure per band
    k_min, for every LES time step dt_les = f * dt_dns in dt_factors (f must
    divide `every`; the LES grid is 16x coarser, so f up to ~16 keeps its CFL
    number below the DNS's).  Per report: the LES and filtered-DNS spectra for
    k <= KMAX, TKE, enstrophy, and the wall-clock of every solver over the
    same simulated time."""
    out = []
    variants = []   # (name, band or None, dt factor)
    for f in dt_factors:
        suffix = "" if f == 1 else f"_dt{f}"
        variants.append(("none" + suffix, None, f))
        variants += [(f"closure_k{b:g}" + suffix, b, f) for b in bands]
    names = [v[0] for v in variants]
    for s in seeds:
        with S.Spectral2D(n_dns, nu=nu) as dns, S.Spectral2D(n_les, nu=nu) as filt:
            les = {nm: S.Spectral2D(n_les, nu=nu, precision=les_precision) for nm in names}
            dns.set_turbulent_velocity(seed=s, spectrum="k4gauss", k0=10.0, tke=0.5)
            dt = dns.compute_time_step(cfl)
            for nm, band, _ in variants:
                S.filter_state(dns, les[nm])
                if band is not None:
                    S.les_set_closure(les[nm], net)
            rec = {"seed": s, "dt": dt, "t": [], "E": {nm: [] for nm in ["dns"] + names},
                   "tke": {nm: [] for nm in ["dns"] + names}, "enst": {nm: [] for nm in ["dns"] + names}}
            wall = {nm: 0.0 for nm in ["dns"] + names}
            for done in range(0, steps, every):
                n = min(every, steps - done)
                dns.synchronize()
                a = time.perf_counter()
                dns.integrate_steps(n, dt)
                dns.synchronize()
                wall["dns"] += time.perf_counter() - a
                for nm, band, f in variants:
                    h = les[nm]
                    if band is not None:   # the band is read when the step's graph is built
                        net.band = band
                    h.synchronize()
                    a = time.perf_counter()
                    S.les_integrate_steps(h, n // f, dt * f)
                    h.synchronize()
                    wall[nm] += time.perf_counter() - a
                S.filter_state(dns, filt)
                rec["t"].append((done + n) * dt)
                for nm, h in [("dns", filt)] + list(les.items()):
                    E, tke, z = _spectrum(h)
                    rec["E"][nm].append(E[:KMAX + 1].tolist())
                    rec["tke"][nm].append(tke)
                    rec["enst"][nm].append(z)
            for nm, band, _ in variants:
                les[nm].check_finite()
                if band is not None:
                    S.les_set_closure(les[nm], None)
                les[nm].close()
            rec["ms_per_step"] = {nm: 1e3 * v / steps for nm, v in wall.items()}   # per DNS step of time
            rec["summary"] = {nm: _summary([rec], nm) for nm in names}
            for nm in names:
                rec["summary"][nm]["speedup_vs_dns"] = wall["dns"] / wall[nm]
            log(f"seed {s}: " + ", ".join(f"{nm} {rec['summary'][nm]['mean_rel_err_time_avg']:.3f}"
                                          for nm in names))
            out.append(rec)
    return out


def spectrum_errors(E_les, E_dns):
    """The closure's accuracy metric for one seed: E(k) of the LES and of the
    filtered DNS, each averaged over the report times (rows; columns k = 0 ..
    KMAX), then the relative error per k for 1 <= k <= KMAX.  Returns (mean
    over k, max over k)."""
    k = slice(1, KMAX + 1)
    a = np.mean(np.asarray(E_les, dtype=np.float64), axis=0)[k]
    b = np.mean(np.asarray(E_dns, dtype=np.float64), axis=0)[k]
    e = _rel_err(a, b)
    return float(e.mean()), float(e.max())


def _summary(recs, nm):
    """Spectrum errors of variant nm against the filtered DNS for 1 <= k <= KMAX.
    The headline metric is per seed and time-averaged (spectrum_errors: the
    time-averaged spectra compared per k, mean and max over k, then the worst
    seed); beside it, the errors of the instantaneous spectra (mean over k,
    then over report times, and at the final time) and of the seed-averaged
    spectra (the ensemble statistics of the held-out seeds), plus the final
    enstrophy error."""
    k = slice(1, KMAX + 1)
    per = np.array([[_rel_err(np.array(e)[k], np.array(f)[k]) for e, f in zip(r["E"][nm], r["E"]["dns"])]
                    for r in recs])                        # seeds x times x k
    Em = np.mean([np.array(r["E"][nm]) for r in recs], axis=0)[:, k]
    Ed = np.mean([np.array(r["E"]["dns"]) for r in recs], axis=0)[:, k]
    ens = _rel_err(Em, Ed)                                 # times x k
    zf = np.array([r["enst"][nm][-1] / r["enst"]["dns"][-1] - 1.0 for r in recs])
    ta = [spectrum_errors(r["E"][nm], r["E"]["dns"]) for r in recs]
    return {"per_seed_time_avg_spectrum_mean_rel_err": {str(r["seed"]): m for r, (m, _) in zip(recs, ta)},
            "per_seed_time_avg_spectrum_max_rel_err": {str(r["seed"]): x for r, (_, x) in zip(recs, ta)},
            "worst_seed_time_avg_spectrum_mean_rel_err": max(m for m, _ in ta),
            "worst_seed_time_avg_spectrum_max_rel_err": max(x for _, x in ta),
            "mean_rel_err_time_avg": float(per.mean()),
            "mean_rel_err_final": float(per[:, -1].mean()),
            "max_rel_err_final": float(per[:, -1].max()),
            "seed_avg_mean_rel_err_time_avg": float(ens.mean()),
            "seed_avg_mean_rel_err_final": float(ens[-1].mean()),
            "seed_avg_max_rel_err_time_avg": float(ens.mean(axis=0).max()),
            "enstrophy_rel_err_final": float(np.abs(zf).mean())}


def save_weights(net, path):
    np.savez_compressed(path, params=net.get_params(), scales=net.get_scales(), grid=net.grid,
                        band=net.band)


def load_weights(net, path):
    d = np.load(path)
    net.set_params(d["params"])
    net.set_scales(d["scales"])
    net.band = float(d["band"]) if "band" in d else 0.0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-dns", type=int, default=2048)
    ap.add_argument("--n-les", type=int, default=128)
    ap.add_argument("--nu", type=float, default=1e-4)
    ap.add_argument("--cfl", type=float, default=0.5)
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--snaps", type=int, default=500)
    ap.add_argument("--every", type=int, default=40)
    ap.add_argument("--spinup", type=int, default=0)
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-min-frac", type=float, default=0.05)
    ap.add_argument("--bands", type=str, default="0,4,8,16",
                    help="candidate k_min of the closure term, chosen on --val-seed")
    ap.add_argument("--val-seed", type=int, default=10)
    ap.add_argument("--eval-seeds", type=str, default="8,9")
    ap.add_argument("--eval-steps", type=int, default=20000)
    ap.add_argument("--eval-every", type=int, default=1000)
    ap.add_argument("--les-precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--dt-factors", type=str, default="1",
                    help="LES time steps as multiples of the DNS's, e.g. 1,10")
    ap.add_argument("--weights", default=None)
    ap.add_argument("--load", default=None, help="skip data and training; use these weights")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    grid = 3 * a.n_les // 2
    res = {"config": vars(a)}
    bands = [float(b) for b in a.bands.split(",") if b]
    with S.ClosureNet(grid, max_batch=a.batch, seed=0) as net:
        if a.load:
            load_weights(net, a.load)
            bands = [net.band]
        else:
            seeds = list(range(a.train_seeds))
            dts, tg = generate(net, seeds, a.n_dns, a.n_les, a.nu, a.cfl, a.spinup, a.snaps, a.every)
            rms = net.dataset_stats()
            net.set_scales(rms)
            hist, tt = train(net, net.dataset_size, a.epochs, a.batch, a.lr, a.lr_min_frac)
            res.update({"pairs": net.dataset_size, "data_seconds": tg, "train_seconds": tt,
                        "rms": rms.tolist(), "loss_history": hist})
            # the band is chosen on a validation seed that is neither trained on nor evaluated
            if len(bands) > 1:
                val = evaluate(net, [a.val_seed], a.n_dns, a.n_les, a.nu, a.cfl, a.eval_steps,
                               a.eval_every, bands, a.les_precision)
                score = {b: val[0]["summary"][f"closure_k{b:g}"]["mean_rel_err_time_avg"] for b in bands}
                best = min(bands, key=lambda b: score[b])
                res["band_selection"] = {"val_seed": a.val_seed, "score": {f"{b:g}": v for b, v in score.items()},
                                         "k_min": best}
                print(f"band chosen on seed {a.val_seed}: k_min = {best:g} ({score})")
                bands = sorted({0.0, best})
                net.band = best
            else:
                net.band = bands[0]
            if a.weights:
                save_weights(net, a.weights)
        ev = [int(s) for s in a.eval_seeds.split(",") if s]
        factors = [int(f) for f in a.dt_factors.split(",") if f]
        recs = evaluate(net, ev, a.n_dns, a.n_les, a.nu, a.cfl, a.eval_steps, a.eval_every, bands,
                        a.les_precision, factors)
        res["eval"] = recs
        res["eval_summary"] = {nm: _summary(recs, nm) for nm in recs[0]["summary"]}
        for nm in recs[0]["summary"]:
            res["eval_summary"][nm]["speedup_vs_dns"] = float(np.mean(
                [r["summary"][nm]["speedup_vs_dns"] for r in recs]))
        res["k_min"] = net.band
        print("eval summary:", json.dumps(res["eval_summary"]))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f)
    return res


if __name__ == "__main__":
    main()
