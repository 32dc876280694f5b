"""Run one workload of the engine for a profiler (ncu) to capture, without timing or checks.

    python -m ekgsim_gb300.profile_case ca [--grid N]          heart set-up of an N^3 ellipsoid
                                                               (activation-time relaxation, de-duplication)
    python -m ekgsim_gb300.profile_case batched [--sims S] [--passes P] [--moved-all] [--free-k1]
                                                               S-simulation batched passes on the
                                                               160^3 heart of the batched workload
                                                               (--free-k1: k1 differs between the
                                                               simulations, the per-simulation form)

The workloads are the seeded synthetic ones of ekgsim_gb300.synth.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import engine as E
from . import synth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["ca", "batched"])
    ap.add_argument("--grid", type=int, default=160)
    ap.add_argument("--sims", type=int, default=256)
    ap.add_argument("--passes", type=int, default=3)
    ap.add_argument("--moved-all", action="store_true")
    ap.add_argument("--free-k1", action="store_true")
    a = ap.parse_args()
    eng = E.Engine(0)
    if a.case == "ca":
        c = synth.config(2)
        f = a.grid / 160.0
        base = c["spec"]
        spec = synth.HeartSpec(a.grid, tuple(x * f for x in base.semi_axes), base.wall * f, 3, [1, 2, 2], 12, 120.0 * f,
                               seed=base.seed)
        grid = synth.ellipsoid_heart(spec)
        tm = synth.transfer_matrix(3, spec.delays)
        leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
        h = E.Heart.create(eng, grid, tm, leads, "3D4", 0.0, 600.0, 1.0)
        print(f"ca: {a.grid}^3, {h.info.ca_rounds} rounds, {h.info.ca_ms:.3f} ms")
        h.close()
    else:
        c = synth.config(2)
        spec, steps = c["spec"], c["steps"]
        grid = synth.ellipsoid_heart(spec)
        tm = synth.transfer_matrix(3, spec.delays)
        leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
        h = E.Heart.create(eng, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
        h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                   [t for t in synth.analytic_target(spec.n_leads, steps, spec.seed + 999)], mid_position=0.6)
        genes = np.stack([synth.genes_for(spec, r, 2) for r in range(a.sims)])
        if a.moved_all:
            rng = np.random.Generator(np.random.PCG64(spec.seed + 77))
            genes[:, 12:] = -50.0 + 100.0 * rng.random((a.sims, 2 * spec.n_leads))
        lk = np.stack([E.layer_aps(h._cfg, spec.n_layers, g[:12])[0] for g in genes])
        if a.free_k1:
            lk[:, :, 1] *= 1.0 + 1e-3 * np.arange(a.sims)[:, None]  # k1 as a free gene
        moved = np.stack([E.move_leads(leads, g[12:].reshape(-1, 2)) for g in genes])
        bm = h.benchmark(lk, moved, warmup=1, iters=a.passes)
        it = a.passes
        print(f"{'batched' if bm['batched'] else 'per-simulation'} form: {a.sims} sims, "
              f"{bm['total_ms'] / it:.3f} ms per pass (prep {bm['prep_ms'] / it:.3f}, contract "
              f"{bm['contract_ms'] / it:.3f}, tail {bm['tail_ms'] / it:.3f}, operand {bm['operand_ms'] / it:.3f})")
        h.close()
    eng.close()


if __name__ == "__main__":
    main()
