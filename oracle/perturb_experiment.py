"""How far one ulp in pow and log10 moves the column step (TEST INFRASTRUCTURE).

The kernels and the oracle share one binary64 log/exp/pow (clm_math.h), so they agree
bit for bit; the reference computes with Julia's own ^ and log10, which cannot run
here.  This experiment bounds what that difference can do: it runs the oracle's column
step (soil_temperature!, set_soil_water_fractions!, soil_water!) for 48 steps on the
three synthetic workloads, once as built and once with the hot path's pow and log10
results perturbed (the oracle's sensitivity hook, clm_oracle.c):

  ulp-all     every result moved by +-1 ulp (two libraries that never agree);
  ulp-1e-3    one result in 10^3 moved by +-1 ulp (two nearly correctly rounded
              libraries: this one misrounds about 4 in 10^4 random cases);
  ulp-1e-4    one result in 10^4;
  old-pow     the previous library (binary64 log, errors up to |y log x| ulp).

For each it reports the share of columns whose final imelt flags or substep counts
differ from the unperturbed run, and whose temperature, water or ice leave the 1e-10
relative tolerance.  Usage (from the repository root):

  python oracle/perturb_experiment.py [--nc 4096] [--steps 48] [--threads N]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, os.path.join(ROOT, "clm.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from clmgb import synth  # noqa: E402
from oracle import oracle as orc  # noqa: E402

MODES = (("ulp-all", 1, 0.0), ("ulp-1e-3", 2, 1e-3), ("ulp-1e-4", 2, 1e-4), ("old-pow", 3, 0.0))
FIELDS = ("t_soisno", "h2osoi_liq", "h2osoi_ice")


def run(cfg_id, nc, steps, seed, threads, mode=0, frac=0.0, salt=0):
    wl = synth.make_workload(cfg_id, nc=nc, seed=seed, nsteps=steps)
    st = wl.state
    G, I = wl.forcing_block(range(steps))
    orc.set_perturbation(mode, frac, salt)
    try:
        status = orc.run_steps(st, wl.dtime, G, I, nthreads=threads)
    finally:
        orc.set_perturbation(0)
    return st, status


def differ(a, b, rtol=1e-10, atol=1e-12):
    """Per-column flags: imelt differs, substep count differs, a field beyond tolerance;
    and the largest relative difference of the fields."""
    im = np.any(a["imelt"] != b["imelt"], axis=0)
    ns = a["num_substeps"] != b["num_substeps"]
    tol = np.zeros(a.nc, dtype=bool)
    worst = 0.0
    for k in FIELDS:
        x, y = a[k], b[k]
        err = np.abs(x - y)
        tol |= np.any(err > rtol * np.abs(y) + atol, axis=0)
        with np.errstate(invalid="ignore", divide="ignore"):
            rel = np.where(err > 0, err / np.maximum(np.abs(y), 1e-300), 0.0)
        worst = max(worst, float(np.nanmax(rel)))
    return im, ns, tol, worst


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nc", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    print("| workload | perturbation | imelt differs | substeps differ | beyond 1e-10 | max rel diff |")
    print("|---|---|---|---|---|---|")
    for cfg_id in (0, 1, 2):
        base, _ = run(cfg_id, args.nc, args.steps, 100 + cfg_id, args.threads)
        for name, mode, frac in MODES:
            st, _ = run(cfg_id, args.nc, args.steps, 100 + cfg_id, args.threads, mode, frac, salt=12345)
            im, ns, tol, worst = differ(st, base)
            n = float(base.nc)
            print("| config %d (%d columns, %d steps) | %s | %.2f %% | %.2f %% | %.2f %% | %.1e |"
                  % (cfg_id, base.nc, args.steps, name, 100 * im.sum() / n, 100 * ns.sum() / n,
                     100 * tol.sum() / n, worst))


if __name__ == "__main__":
    main()
