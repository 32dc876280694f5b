"""Benchmark: simulated ECGs per second on one GB300 (replicas on N GPUs), JSON line on stdout.

Workload (default): the batched configuration -- one resident 160^3 ellipsoid heart (wall 14,
3 layers, delays {1,2,2}), 12 leads on a radius-120 sphere, 600 steps of 1 ms, 256 seeded
16-gene parameter vectors per step.  A step is one batched evaluation of those 256 vectors.

  value      simulations/s from CUDA events around the device passes, inputs resident in HBM
  e2e        simulations/s through the public C ABI (ekg_eval_batch_submit / _wait, two batches in
             flight; the synchronous ekg_eval_batch rate is beside it): host genes in, host
             criteria + ECGs out, host<->device copies and host gene mapping inside the timed region
  plain      the plain single-simulation form (ekg_eval, one call per simulation) on the same heart
  roofline   the dominant kernel, timed alone with CUDA events: in the batched form the moved-lead
             operand kernel against the measured HBM copy bandwidth (its byte floor; the kernel is
             FP32-issue-bound), with the band GEMM's executed tensor rate beside it; in the
             per-simulation form the band-form contraction against the measured HBM copy
             bandwidth (the bytes it moves), or a dense contraction against the bf16 peak
  cpu_baseline  the reference's CPU algorithm (FP64 port with the reference's cost structure,
             bit-identical results) run as one independent simulation per host core, on a bounded
             sample of the same heart (the first few time steps; cost is linear in steps)

--impl reference runs only that CPU farm (rank 0), on the same workload, metric and unit.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ECG sims/sec & p99 latency, batched vs plain on GB300, ECG rel-L2<=1e-4 vs FP64"


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max-over-ranks for replica runs (torch.distributed gloo on host tensors)."""

    def __init__(self):
        self.rank, self.world, self.local = dist_info()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_heart_spec(name: str):
    from ekgsim_gb300 import synth
    if name == "batched":
        c = synth.config(2)
        return c["spec"], c["steps"], c["batch"], 2, c["name"]
    if name == "bsm":
        c = synth.config(4)
        return c["spec"], c["steps"], c["batch"], 4, c["name"]
    c = synth.config(1)
    return c["spec"], c["steps"], 64, 1, c["name"]


def build_inputs(spec, steps, batch, cfg_index):
    from ekgsim_gb300 import synth
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    leads_zyx = synth.leads(spec, rng)[:, ::-1].copy()
    genes = np.stack([synth.genes_for(spec, r, cfg_index) for r in range(batch)])
    target = synth.analytic_target(spec.n_leads, steps, spec.seed + 999)
    return grid, tm, leads_zyx, genes, target


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per simulation of `kernel` from the committed ncu summary of that workload."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_sim:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def cpu_farm(spec, steps, genes, sample_steps: int, threads: int):
    """The reference's CPU algorithm as a farm of independent single-threaded simulations, one per
    host core, each on the first `sample_steps` steps.  Returns (sims/s, seconds, sample text)."""
    from concurrent.futures import ThreadPoolExecutor
    from ekgsim_gb300 import synth
    from oracle import oracle as O
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    leads_zyx = synth.leads(spec, rng)[:, ::-1].copy()
    at, layer = O.activation(grid, tm)
    jobs = []
    for i in range(threads):
        g = genes[i % len(genes)]
        lk, _, _ = O.layer_aps(spec.n_layers, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX,
                               [5, 6, 7, 8], "endo-mid-epi", 0.6, g[:12])
        moved = O.move_leads(leads_zyx, g[12:12 + 2 * spec.n_leads].reshape(-1, 2))
        jobs.append((lk, moved))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda j: O.run_naive(layer, at, j[0], j[1], "3D4", 0.0, float(steps), 1.0, sample_steps), jobs))
    dt = time.perf_counter() - t0
    per_sim = dt * steps / sample_steps
    sims_per_s = threads / per_sim
    sample = (f"{threads} concurrent single-thread simulations of the {spec.n}^3 heart, first {sample_steps} of "
              f"{steps} steps each ({dt:.1f} s wall), scaled by {steps}/{sample_steps}")
    return sims_per_s, dt, sample


def served_hearts(eng):
    """The four resident hearts of the served configuration (48^3, 96^3, 144^3, 192^3 scaled
    ellipsoids, 3 layers, 12 leads, 600 steps), evaluation settings set."""
    from ekgsim_gb300 import engine as E
    from ekgsim_gb300 import synth
    cfg = synth.config(3)
    hearts, specs = [], []
    for spec in cfg["hearts"]:
        grid = synth.ellipsoid_heart(spec)
        tm = synth.transfer_matrix(spec.n_layers, spec.delays)
        leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
        h = E.Heart.create(eng, grid, tm, leads, "3D4", 0.0, float(cfg["steps"]), 1.0)
        h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                   [t for t in synth.analytic_target(spec.n_leads, cfg["steps"], spec.seed + 999)], mid_position=0.6)
        hearts.append(h)
        specs.append(spec)
    return hearts, specs


def served_stream(srv, ids, specs, rate: float, n: int, seed: int, n_crit: int):
    """One Poisson stream of n requests at `rate` per second over the hearts (uniformly), submitted
    through ekg_server_submit_many as they fall due (the loop wakes every ~50 us) and handed over
    with ekg_server_poll_many.  Latency is the engine's submit -> result time per request."""
    from ekgsim_gb300 import synth
    rng = np.random.Generator(np.random.PCG64(seed))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    which = rng.integers(0, len(ids), size=n).astype(np.int32)
    # 16 README-bounded genes per request, zeros for the displacements of leads 2..11
    genes = np.zeros((n, 12 + 2 * specs[0].n_leads))
    genes[:, :16] = synth.GENE_MIN + (synth.GENE_MAX - synth.GENE_MIN) * rng.random((n, 16))
    hid = np.array([ids[w] for w in which], dtype=np.int32)
    rids = np.zeros(n, dtype=np.uint64)
    sub_t = np.zeros(n)
    t0 = time.perf_counter()
    i = 0
    while i < n:
        now = time.perf_counter() - t0
        j = int(np.searchsorted(arrivals, now, side="right"))
        if j > i:
            rids[i:j] = srv.submit_many(hid[i:j], genes[i:j])
            sub_t[i:j] = now
            i = j
        else:
            time.sleep(min(5e-5, max(0.0, arrivals[i] - now)))
    status, crit, viol, total, batch = srv.poll_many(rids, n_crit, wait_ms=600000)
    assert (status == 0).all(), "served requests failed"
    done_t = sub_t + total / 1000.0
    span = float(done_t.max() - min(arrivals[0], sub_t[0]))
    return {"rate_req_s": rate, "requests": n, "throughput_req_s": n / span,
            "p50_ms": float(np.percentile(total, 50)), "p99_ms": float(np.percentile(total, 99)),
            "mean_batch": float(np.mean(batch))}


def served_run(rates=(500.0, 5e3, 5e4, 2e5, 4e5, 1e6), seconds: float = 1.0, max_requests: int = 200_000,
               seed: int = 3000, max_wait_us: int = 0):
    """Served configuration: Poisson streams of evaluation requests over four resident hearts,
    continuous batching in the engine's request loop (each heart's next pass is prepared and queued
    while its current one runs; with max_wait_us = 0 a pass starts as soon as its heart has nothing on
    the device).  One stream per offered rate; the highest rate saturates the engine, so its
    throughput is the served form's capacity."""
    from ekgsim_gb300 import engine as E
    from ekgsim_gb300 import synth
    eng = E.Engine(0)
    hearts, specs = served_hearts(eng)
    srv = E.Server(eng, max_batch=256, max_wait_us=max_wait_us, keep_ecg=False)
    ids = [srv.add_heart(h) for h in hearts]
    _, nc = hearts[0].eval_shape()
    # warm each heart's batched path (graph capture, buffers) with a few full passes
    for k in range(3):
        hid = np.repeat(np.array(ids, dtype=np.int32), 256)
        g = np.stack([synth.genes_for(specs[i // 256], 20_000 + k * 1024 + i, 3) for i in range(hid.size)])
        st = srv.poll_many(srv.submit_many(hid, g), nc, wait_ms=600000)[0]
        assert (st == 0).all()
    sweep = []
    for r_i, rate in enumerate(rates):
        n = int(min(max_requests, max(200, rate * seconds)))
        sweep.append(served_stream(srv, ids, specs, rate, n, seed + r_i, nc))
    srv.close()
    for h in hearts:
        h.close()
    eng.close()
    sat = max(sweep, key=lambda d: d["throughput_req_s"])
    return {"hearts": [s.n for s in specs], "max_batch": 256, "max_wait_us": max_wait_us,
            "form": "per-heart dispatchers, two passes in flight per heart, criteria only (no ECG copies)",
            "sweep": sweep, "saturated": sat}


def parity_check(E, eng, grid, tm, leads_zyx, spec, steps, genes, target, ecg, heart, lk, moved, n_oracle):
    """Parity of the timed batch's results, by a stated policy:
    - every result against the engine's per-simulation form (a second heart on an engine with the
      batched form off: band-form FP32 contraction, a different algorithm from the batched form's
      static-lead basis and tensor-core band GEMM), ECG rel-L2 per result;
    - n_oracle results spread over the batch (first, last, middle, seeded random others) against
      the FP64 oracle (the reference's algorithm, pinned bit for bit to the compiled reference);
    - activation times of the heart against the oracle's, bitwise."""
    from oracle import oracle as O
    batch = len(genes)
    at_ref, layer = O.activation(grid, tm)
    at_gpu = heart.activation()
    mism = int(np.count_nonzero(at_gpu.view(np.int64) != at_ref.view(np.int64)))
    pick = sorted(set([0, batch - 1, batch // 2] + [int(x) for x in np.random.Generator(
        np.random.PCG64(7)).choice(batch, size=min(batch, max(0, n_oracle - 3)), replace=False)]))[:max(1, n_oracle)]
    rels = []
    for i in pick:
        ref = O.run(layer, at_ref, lk[i], moved[i], "3D4", 0.0, float(steps), 1.0)
        rels.append(float(np.linalg.norm(ecg[i] - ref) / np.linalg.norm(ref)))
    os.environ["EKG_BATCHED"] = "0"
    try:
        eng2 = E.Engine(0)
    finally:
        os.environ.pop("EKG_BATCHED", None)
    h2 = E.Heart.create(eng2, grid, tm, leads_zyx, "3D4", 0.0, float(steps), 1.0)
    h2.set_eval(*heart.eval_args[0], **heart.eval_args[1])
    _, _, ecg2 = h2.eval_batch(genes, want_ecg=True)
    cross = [float(np.linalg.norm(ecg[i] - ecg2[i]) / np.linalg.norm(ecg2[i])) for i in range(batch)]
    h2.close()
    eng2.close()
    return {"policy": "every result vs the per-simulation form; a spread sample vs the FP64 oracle; activation "
                      "times bitwise", "ecg_rel_l2_max": max(rels), "checked_sims": len(rels), "oracle_sims": pick,
            "cross_form_rel_l2_max": max(cross), "cross_checked": batch, "at_mismatch": mism,
            "tolerance": 1e-4}


def all_leads_moved(E, heart, leads_zyx, spec, steps, batch, cfg_index, grid, tm, iters, no_tune):
    """The same batched workload with displacement genes for all leads (the reference's normal
    "optimize measuring points" case: 12 + 2L genes, sim.cpp:835), so every lead's field is
    evaluated per simulation: device simulations/s with inputs resident, and two results against the
    FP64 oracle."""
    from ekgsim_gb300 import synth
    from oracle import oracle as O
    rng = np.random.Generator(np.random.PCG64(spec.seed + 77))
    genes = np.stack([synth.genes_for(spec, r, cfg_index) for r in range(batch)])
    genes[:, 12:] = -50.0 + 100.0 * rng.random((batch, 2 * spec.n_leads))
    cfg = heart._cfg
    lk = np.stack([E.layer_aps(cfg, spec.n_layers, g[:12])[0] for g in genes])
    moved = np.stack([E.move_leads(leads_zyx, g[12:].reshape(-1, 2)) for g in genes])
    tuned = heart.tune(lk, moved, reps=2) if not no_tune else None
    heart.benchmark(lk, moved, warmup=3, iters=1)
    bm = heart.benchmark(lk, moved, warmup=0, iters=iters)
    ms = bm["total_ms"] / iters
    ecg = heart.eval_batch(genes, want_ecg=True)[2]
    at, layer = O.activation(grid, tm)
    rels = []
    for i in (0, batch - 1):
        ref = O.run(layer, at, lk[i], moved[i], "3D4", 0.0, float(steps), 1.0)
        rels.append(float(np.linalg.norm(ecg[i] - ref) / np.linalg.norm(ref)))
    return {"moved_leads": int(bm["moved_leads"]), "sims_per_s": batch / (ms / 1000.0), "ms_per_step": ms,
            "operand_ms": bm["operand_ms"] / iters, "contract_ms": bm["contract_ms"] / iters, "tuned": tuned,
            "ecg_rel_l2_max": max(rels), "checked_sims": len(rels)}


def free_k1(E, heart, leads_zyx, spec, steps, batch, cfg_index, grid, tm, iters, target):
    """The same workload with k1 (the upstroke rate) a free gene, so every simulation has its own
    k1 and the batch takes the per-simulation form (moved leads' field, band contraction, chunk
    reduction): device simulations/s with inputs resident, and two results against the FP64 oracle.
    Leaves the heart's evaluation settings with k1 free."""
    from ekgsim_gb300 import synth
    from oracle import oracle as O
    free = [1, 5, 6, 7, 8]
    heart.set_eval([synth.BASE_AP] * spec.n_layers, synth.K_MIN, synth.K_MAX, free, [t for t in target],
                   mid_position=0.6)
    ng, _ = heart.eval_shape()
    lo, hi = heart.gene_bounds()
    rng = np.random.Generator(np.random.PCG64(spec.seed + 91))
    genes = lo + (hi - lo) * rng.random((batch, ng))
    genes[:, 15:] = np.stack([synth.genes_for(spec, r, cfg_index)[12:] for r in range(batch)])
    cfg = heart._cfg
    lk = np.stack([E.layer_aps(cfg, spec.n_layers, g[:15])[0] for g in genes])
    moved = np.stack([E.move_leads(leads_zyx, g[15:].reshape(-1, 2)) for g in genes])
    heart.benchmark(lk, moved, warmup=3, iters=1)
    bm = heart.benchmark(lk, moved, warmup=0, iters=iters)
    ms = bm["total_ms"] / iters
    ecg = heart.eval_batch(genes, want_ecg=True)[2]
    at, layer = O.activation(grid, tm)
    rels = []
    for i in (0, batch - 1):
        ref = O.run(layer, at, lk[i], moved[i], "3D4", 0.0, float(steps), 1.0)
        rels.append(float(np.linalg.norm(ecg[i] - ref) / np.linalg.norm(ref)))
    return {"form": "batched" if bm["batched"] else "per-simulation", "free_k": free,
            "moved_leads": int(bm["moved_leads"]), "sims_per_s": batch / (ms / 1000.0), "ms_per_step": ms,
            "lead_field_ms": bm["prep_ms"] / iters, "contract_ms": bm["contract_ms"] / iters,
            "tail_ms": bm["tail_ms"] / iters, "ecg_rel_l2_max": max(rels), "checked_sims": len(rels)}


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def workload_config(spec, steps, batch, wname, n_voxels, n_aps, world):
    """The `config` object both arms print, so that their lines describe the same workload."""
    return {"workload": wname, "grid": spec.n, "voxels": int(n_voxels), "aps": int(n_aps), "leads": spec.n_leads,
            "steps": steps, "batch": batch, "layers": spec.n_layers,
            "l2": "inputs larger than L2 (per-step lead fields and partials exceed 129 MB)",
            "parallelism": f"replicas{world}"}


def run_reference(args):
    """The reference's CPU algorithm (the oracle's port with the reference's own cost structure:
    every cell and neighbour AP evaluated per step, simlib/simulator.cpp:452-550) as a farm of P
    concurrent single-threaded simulations, P = host cores, as the reference's MPI farm runs
    independent evaluations.  The K timed steps are consecutive slices of the time axis of the
    same P simulations, so together they run P complete simulations of every time step: nothing is
    extrapolated.  The W warm-up steps each run one time step of every simulation first."""
    d = Dist()
    if d.rank != 0:
        d.close()
        return
    from concurrent.futures import ThreadPoolExecutor
    from ekgsim_gb300 import synth
    from oracle import oracle as O
    spec, steps, batch, cfg_index, wname = make_heart_spec(args.workload)
    cores = host_cores()
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    leads_zyx = synth.leads(spec, rng)[:, ::-1].copy()
    at, layer = O.activation(grid, tm)
    n_vox = int(np.count_nonzero(layer))
    n_aps = int(O.ap_indices(layer, at)[0].max() + 1)
    jobs = []
    for i in range(cores):
        g = synth.genes_for(spec, i, cfg_index)
        lk, _, _ = O.layer_aps(spec.n_layers, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX,
                               [5, 6, 7, 8], "endo-mid-epi", 0.6, g[:12])
        jobs.append((lk, O.move_leads(leads_zyx, g[12:12 + 2 * spec.n_leads].reshape(-1, 2))))

    def farm(k0, k1):
        with ThreadPoolExecutor(max_workers=cores) as ex:
            list(ex.map(lambda j: O.run_naive_range(layer, at, j[0], j[1], "3D4", 0.0, float(steps), 1.0, k0, k1),
                        jobs))

    for w in range(args.warmup):
        farm(w % steps, w % steps + 1)
    bounds = [round(steps * i / args.steps) for i in range(args.steps + 1)]
    step_s = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        farm(bounds[i], bounds[i + 1])
        step_s.append(time.perf_counter() - t0)
    total = sum(step_s)
    value = cores / total
    sample = (f"{cores} concurrent single-thread simulations of the {spec.n}^3 heart (the reference's per-voxel "
              f"cost structure), all {steps} time steps: the {args.steps} timed steps are consecutive slices of "
              f"the time axis of the same simulations ({total:.1f} s wall in all); nothing is extrapolated")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "sims/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(spec, steps, batch, wname, n_vox, n_aps, args.gpus),
        "cpu_baseline": {"value": value, "unit": "sims/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "sims/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_s": {"min": min(step_s), "max": max(step_s)},
    }
    print(json.dumps(line), flush=True)
    d.close()


def run_ours(args):
    d = Dist()
    from ekgsim_gb300 import engine as E
    from ekgsim_gb300 import synth
    spec, steps, batch, cfg_index, wname = make_heart_spec(args.workload)
    if args.batch:
        batch = args.batch
    grid, tm, leads_zyx, genes, target = build_inputs(spec, steps, batch, cfg_index)
    eng = E.Engine(d.local)
    # a small heart first, so that the measured heart's set-up does not include module loading
    ws = synth.small_spec(16)
    E.Heart.create(eng, synth.ellipsoid_heart(ws), synth.transfer_matrix(3, ws.delays), np.array([[40.0, 40.0, 40.0]]),
                   "3D4", 0.0, 10.0, 1.0).close()
    t0 = time.perf_counter()
    heart = E.Heart.create(eng, grid, tm, leads_zyx, "3D4", 0.0, float(steps), 1.0)
    setup_s = time.perf_counter() - t0
    heart.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target],
                   mid_position=0.6, optimize_points=True, comparison_mode=2)
    info = heart.info
    # per-simulation layer APs and moved leads (host, as the evaluation does)
    cfg = heart._cfg
    lk = np.stack([E.layer_aps(cfg, info.n_layers, g[:12])[0] for g in genes])
    moved = np.stack([E.move_leads(leads_zyx, g[12:].reshape(-1, 2)) for g in genes])

    # the autotuner picks the batched form's launch shapes for this pass shape (timed on the heart)
    tuned = heart.tune(lk, moved, reps=3) if not args.no_tune else None

    # device-only throughput (inputs resident)
    for _ in range(1):
        heart.benchmark(lk, moved, warmup=args.warmup, iters=1)
    d.barrier()
    clocks = ClockSampler(d.local)
    clocks.start()
    bm = heart.benchmark(lk, moved, warmup=0, iters=args.steps)
    clk = clocks.stop()
    dev_s = d.max(bm["total_ms"] / 1000.0)
    d.barrier()
    value = d.world * batch * args.steps / dev_s

    # end to end through the public API: genes in host memory, criteria + ECGs out to host buffers
    # the caller allocated once.  Synchronous calls (ekg_eval_batch), and queued calls
    # (ekg_eval_batch_submit / _wait) with two batches in flight so that the host part of the next
    # batch overlaps the device pass of the current one (output buffers page-locked); the headline
    # e2e is the queued form
    ng, nc = heart.eval_shape()
    outs = [(np.empty((batch, nc)), np.empty(batch), np.empty((batch, info.n_leads, steps))) for _ in range(2)]
    for _ in range(args.warmup):
        heart.eval_batch(genes, want_ecg=True, out=outs[0])
    d.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        crit, viol, ecg = heart.eval_batch(genes, want_ecg=True, out=outs[0])
    e2e_sync = d.world * batch * args.steps / d.max(time.perf_counter() - t0)
    for o in outs:
        for a in o:
            E.host_register(a)
    for k in range(args.warmup):
        heart.eval_batch_wait(heart.eval_batch_submit(genes, outs[k % 2], want_ecg=True))
    d.barrier()
    t0 = time.perf_counter()
    prev = None
    for k in range(args.steps):
        t = heart.eval_batch_submit(genes, outs[k % 2], want_ecg=True)
        if prev is not None:
            heart.eval_batch_wait(prev)
        prev = t
    heart.eval_batch_wait(prev)
    e2e_s = d.max(time.perf_counter() - t0)
    e2e = d.world * batch * args.steps / e2e_s
    for o in outs:
        for a in o:
            E.host_unregister(a)
    ng, nc = heart.eval_shape()
    h2d = batch * (info.n_layers * 9 + info.n_leads * 3) * 8
    d2h = batch * (info.n_leads * steps * 8 + min(info.n_leads, len(target)) * 2 * 8)

    # plain form: one simulation per call, latency distribution
    lat = []
    for i in range(args.warmup + max(20, args.plain_calls)):
        t1 = time.perf_counter()
        heart.eval(genes[i % batch])
        if i >= args.warmup:
            lat.append(time.perf_counter() - t1)
    lat = np.array(lat) * 1000.0
    plain = {"sims_per_s": float(1000.0 / lat.mean()), "p50_ms": float(np.percentile(lat, 50)),
             "p99_ms": float(np.percentile(lat, 99)), "calls": int(lat.size)}

    # roofline of the dominant kernel, live from CUDA events on the launching stream
    bf16, hbm, src = peaks()
    if bm["batched"] and bm["moved_leads"] > 0:
        # moved-lead operand kernel: FP32 field evaluation (issue-bound); its HBM floor is the bytes
        # it has to move (BF16 hi+lo tile rows and steady sums out, voxel geometry in)
        op_s = bm["operand_ms"] / 1000.0 / args.steps
        tr = profiled_traffic("k_batch_lead_field", wname)
        achieved = bm["operand_bytes"] / op_s / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": tr * batch if tr is not None else None, "peak_source": src,
                "kernel": "k_batch_lead_field", "launch_ms": op_s * 1000.0,
                "algorithmic_bytes": bm["operand_bytes"],
                "note": "FP32 + SFU issue-bound field evaluation (one rsqrt per interior voxel and lead, one more "
                        "per absent neighbour of a boundary voxel with few absent, nine for the other boundary "
                        "voxels); the HBM figure is the kernel's byte floor"}
        gemm_s = bm["contract_ms"] / 1000.0 / args.steps
        roof["gemm"] = {"kernel": "k_batch_umma", "bound": "tensor", "launch_ms": gemm_s * 1000.0,
                        "executed_tflops": bm["gemm_flops"] / gemm_s / 1e12 if gemm_s > 0 else None,
                        "peak": bf16, "frac": bm["gemm_flops"] / gemm_s / 1e12 / bf16 if gemm_s > 0 else None,
                        "note": "band GEMM, three BF16 products per K step (hi/lo split), FP32 accumulation"}
    elif bm["band_bytes"] > 0:
        # per-simulation form, band-form contraction on the CUDA cores: bound by the bytes it moves
        # (W' read, per-chunk FP64 partial sums written)
        contract_s = bm["contract_ms"] / 1000.0 / args.steps
        kernel = "k_contract_band"
        achieved = bm["band_bytes"] / contract_s / 1e9
        tr = profiled_traffic(kernel, wname)
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": tr * batch if tr is not None else None, "peak_source": src, "kernel": kernel,
                "launch_ms": contract_s * 1000.0, "algorithmic_bytes": bm["band_bytes"],
                "note": "zero / steady / band steps per chunk; the band is evaluated directly in FP32"}
    else:
        contract_s = bm["contract_ms"] / 1000.0 / args.steps  # one launch per step
        kernel = "k_contract_umma"
        alg_flops = 2.0 * info.n_leads * 3 * info.n_voxels * steps * batch
        exec_flops = 3 * 2.0 * (-(-info.n_leads // 16) * 16) * info.n_aps * steps * batch
        achieved = alg_flops / contract_s / 1e12
        tr = profiled_traffic(kernel, wname)
        roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16,
                "traffic": tr * batch if tr is not None else None, "peak_source": src, "kernel": kernel,
                "launch_ms": contract_s * 1000.0, "executed_tflops": exec_flops / contract_s / 1e12,
                "note": "algorithmic flops 2 x L x 3V x T per simulation"}

    line = {
        "metric": METRIC, "value": value, "unit": "sims/s", "n_gpus": d.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": bm["total_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16x3", "data": "synthetic",
        "config": workload_config(spec, steps, batch, wname, info.n_voxels, info.n_aps, d.world),
        "heart": {"setup_s": setup_s, "ca_rounds": int(info.ca_rounds)},
        "e2e": {"value": e2e, "unit": "sims/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "form": "queued batched calls, two in flight", "sync_value": e2e_sync},
        "plain": plain,
        "batched_over_plain": value / plain["sims_per_s"],
        "form": "separable batched" if bm["batched"] else "per-simulation",
        "device_ms": {"prep": bm["prep_ms"] / args.steps, "operand": bm["operand_ms"] / args.steps,
                      "contract": bm["contract_ms"] / args.steps, "tail": bm["tail_ms"] / args.steps},
        "roofline": roof,
        # the activation-time relaxation (once per heart): N^3 x 1 B layers in + N^3 x 8 B times out;
        # latency-bound (one dependent launch per time bucket), so the fraction is its byte floor
        "ca": {"kernel": "k_ca_bucket" if info.ca_buckets else "k_ca_round_list", "steps": int(info.ca_rounds),
               "form": "time buckets" if info.ca_buckets else "tile rounds", "ms": info.ca_ms,
               "algorithmic_bytes": 9 * int(info.n_cells),
               "achieved_gbs": 9 * info.n_cells / (info.ca_ms / 1000.0) / 1e9 if info.ca_ms > 0 else None,
               "frac": 9 * info.n_cells / (info.ca_ms / 1000.0) / 1e9 / hbm if info.ca_ms > 0 else None},
        # the dense lead contraction's algorithmic flops (2 x L x 3V x T per simulation) over the
        # whole device step; the engine does not perform that contraction (W-form over de-duplicated
        # APs, static-lead basis, band split), so this rate can exceed the tensor peak
        "contraction_equivalent": {"flops_per_sim": 2.0 * info.n_leads * 3 * info.n_voxels * steps,
                                   "tflops": 2.0 * info.n_leads * 3 * info.n_voxels * steps * batch * args.steps
                                   / (bm["total_ms"] / 1000.0) / 1e12},
        "tuned": tuned,
        "gpu_launches": int(bm["launches"]) * args.steps,
        "clocks": clk,
    }
    if d.rank == 0 and not args.no_check:
        line["parity"] = parity_check(E, eng, grid, tm, leads_zyx, spec, steps, genes, target, ecg, heart, lk, moved,
                                      args.parity_sims)
    if d.rank == 0 and not args.no_moved_all and args.workload == "batched":
        line["all_leads_moved"] = all_leads_moved(E, heart, leads_zyx, spec, steps, batch, cfg_index, grid, tm,
                                                  args.steps, args.no_tune)
    if d.rank == 0 and not args.no_free_k1 and args.workload == "batched":
        line["free_k1"] = free_k1(E, heart, leads_zyx, spec, steps, batch, cfg_index, grid, tm, args.steps, target)
    if d.rank == 0 and not args.no_served:
        line["served"] = served_run(max_wait_us=args.served_wait_us)
        line["served_over_plain"] = line["served"]["saturated"]["throughput_req_s"] / plain["sims_per_s"]
    if d.rank == 0 and d.world == 1 and not args.no_cpu:
        v, dt, sample = cpu_farm(spec, steps, genes, args.cpu_sample_steps, host_cores())
        line["cpu_baseline"] = {"value": v, "unit": "sims/s", "cores": host_cores(), "kind": "port",
                                "sample": sample}
    if d.rank == 0:
        print(json.dumps(line), flush=True)
    heart.close()
    eng.close()
    d.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "single", "bsm"])
    ap.add_argument("--served-wait-us", type=int, default=0,
                    help="served form: longest a request waits for others to join its pass while its heart is idle")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--plain-calls", type=int, default=50)
    ap.add_argument("--cpu-sample-steps", type=int, default=16)
    ap.add_argument("--parity-sims", type=int, default=8, help="results checked against the FP64 oracle")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the built-in launch shapes")
    ap.add_argument("--no-moved-all", action="store_true", help="skip the all-leads-moved variant")
    ap.add_argument("--no-free-k1", action="store_true", help="skip the free-k1 (per-simulation form) variant")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
