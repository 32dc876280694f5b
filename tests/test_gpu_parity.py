"""GPU parity: the engine (through the C ABI) against the FP64 oracle.

Bars: activation times bit-exact (FP64 equality); ECG relative L2 over leads x steps <= 1e-4
(the FP32-AP / BF16 hi+lo contraction tolerance); criteria within 1e-4 absolute of the oracle's.
"""
import os

import numpy as np
import pytest

from ekgsim_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ECG_TOL = 1e-4


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_heart(engine, spec, steps=300, nhood="3D4", start=0.0, dt=1.0):
    from ekgsim_gb300.engine import Heart
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    leads_zyx = synth.leads(spec, rng)[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads_zyx, nhood, start, steps * dt, dt)
    return h, grid, tm, leads_zyx


def layer_k_for(spec, request=0):
    g = synth.genes_for(spec, request, 0)
    lk, _, _ = O.layer_aps(spec.n_layers, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                           "endo-mid-epi", 0.6, g[:12])
    return lk


@pytest.mark.parametrize("n", [8, 16, 24, 40, 64])
def test_activation_bit_exact(engine, n):
    spec = synth.small_spec(n) if n < 64 else synth.config(0)["spec"]
    h, grid, tm, _ = make_heart(engine, spec, steps=10)
    at_ref, _ = O.activation(grid, tm)
    at = h.activation()
    assert np.array_equal(at.view(np.int64), at_ref.view(np.int64))
    idx_ref, _, _ = O.ap_indices(np.abs(grid), at_ref)
    assert np.array_equal(h.ap_index().ravel(), idx_ref)
    assert h.info.n_aps == idx_ref.max() + 1


def test_activation_bit_exact_128(engine):
    spec = synth.config(1)["spec"]
    h, grid, tm, _ = make_heart(engine, spec, steps=10)
    at_ref, _ = O.activation(grid, tm)
    assert np.array_equal(h.activation().view(np.int64), at_ref.view(np.int64))


def test_activation_unreachable_and_multilayer(engine):
    # two separate blobs, stimulus only in one; 5 layers with mixed delays
    rng = np.random.Generator(np.random.PCG64(5))
    g = np.zeros((20, 22, 18), dtype=np.int32)
    g[2:9, 3:12, 2:10] = rng.integers(1, 6, size=(7, 9, 8))
    g[12:18, 10:20, 8:16] = rng.integers(1, 6, size=(6, 10, 8))
    g[3, 4, 3] = -abs(g[3, 4, 3])
    tm = np.full((12, 12), -1.0)
    tm[1:6, 1:6] = rng.integers(1, 4, size=(5, 5)).astype(float) * 0.5
    from ekgsim_gb300.engine import Heart
    h = Heart.create(engine, g, tm, np.array([[40.0, 40.0, 40.0]]), "3D4", 0.0, 50.0, 1.0)
    at_ref, _ = O.activation(g, tm)
    at = h.activation()
    assert np.array_equal(at.view(np.int64), at_ref.view(np.int64))
    assert (at[12:18, 10:20, 8:16] == 0).all()


def test_activation_2d_grid(engine):
    spec = synth.small_spec(32)
    grid = synth.ellipsoid_heart(spec)[16:17].copy()
    grid[0][grid[0] != 0] = np.abs(grid[0][grid[0] != 0])
    nz = np.argwhere(grid[0] == 1)
    grid[0, nz[0][0], nz[0][1]] = -1
    tm = synth.transfer_matrix(3, [1, 2, 2])
    from ekgsim_gb300.engine import Heart
    h = Heart.create(engine, grid, tm, np.array([[0.0, 40.0, 40.0]]), "2D8", 0.0, 50.0, 1.0)
    at_ref, layer = O.activation(grid, tm)
    assert np.array_equal(h.activation().view(np.int64), at_ref.view(np.int64))
    lk = layer_k_for(spec)
    ecg = h.simulate(lk)
    ref = O.run(layer, at_ref, lk, np.array([[0.0, 40.0, 40.0]]), "2D8", 0.0, 50.0, 1.0)
    assert rel_l2(ecg, ref) <= ECG_TOL


@pytest.mark.parametrize("nhood", ["3D4", "cube", "2D4", "2D8"])
def test_ecg_neighbourhoods(engine, nhood):
    spec = synth.small_spec(24, n_leads=3)
    h, grid, tm, leads = make_heart(engine, spec, steps=250, nhood=nhood)
    at, layer = O.activation(grid, tm)
    lk = layer_k_for(spec, 1)
    ecg = h.simulate(lk)
    ref = O.run(layer, at, lk, leads, nhood, 0.0, 250.0, 1.0)
    assert rel_l2(ecg, ref) <= ECG_TOL


def test_ecg_64_full(engine):
    c = synth.config(0)
    spec = c["spec"]
    h, grid, tm, leads = make_heart(engine, spec, steps=c["steps"])
    at, layer = O.activation(grid, tm)
    for req in range(3):
        g = synth.genes_for(spec, req, 0)
        lk = layer_k_for(spec, req)
        moved = O.move_leads(leads, g[12:16].reshape(2, 2))
        ecg = h.simulate(lk, moved)
        ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(c["steps"]), 1.0)
        assert rel_l2(ecg, ref) <= ECG_TOL, req


def test_ecg_k0_offsets_and_start(engine):
    """Distinct k0 per layer leave a constant term; start != 0 and dt = 0.5 shift the time axis."""
    spec = synth.small_spec(24, n_leads=2)
    h, grid, tm, leads = make_heart(engine, spec, steps=240, start=100.0, dt=0.5)
    at, layer = O.activation(grid, tm)
    lk = layer_k_for(spec, 2)
    lk[:, 0] = [-86.0, -80.0, -90.0]
    ecg = h.simulate(lk)
    ref = O.run(layer, at, lk, leads, "3D4", 100.0, 120.0, 0.5)
    assert rel_l2(ecg, ref) <= ECG_TOL


def _workload(tmp_path, cfg_index, target=None):
    c = synth.config(cfg_index)
    return synth.make_workload(str(tmp_path), c["spec"], c["steps"], target=target), c


def test_eval_matches_oracle_64(engine, tmp_path):
    from ekgsim_gb300.engine import Heart
    w, c = _workload(tmp_path, 0)
    s = O.load_setup(str(tmp_path))
    h = Heart.from_ini(engine, os.path.join(str(tmp_path), "simulator.ini"))
    for req in range(2):
        g = synth.genes_for(c["spec"], req, 0)
        crit_ref, viol_ref, ecg_ref, lk_ref, leads_ref = O.evaluate(s, g)
        crit, viol, ecg, lk, leads = h.eval(g, want_ecg=True)
        assert np.array_equal(lk, lk_ref)
        assert np.array_equal(leads, leads_ref)
        assert viol == viol_ref
        assert rel_l2(ecg, ecg_ref) <= ECG_TOL
        assert np.allclose(crit, crit_ref, rtol=0, atol=1e-4)


def test_batch_matches_single(engine, tmp_path):
    from ekgsim_gb300.engine import Heart
    w, c = _workload(tmp_path, 0)
    h = Heart.from_ini(engine, os.path.join(str(tmp_path), "simulator.ini"))
    genes = np.stack([synth.genes_for(c["spec"], r, 0) for r in range(5)])
    crit_b, viol_b, ecg_b = h.eval_batch(genes, want_ecg=True)
    for i in range(5):
        crit, viol, ecg, _, _ = h.eval(genes[i], want_ecg=True)
        # the batch runs the separable batched form, the single call the per-simulation form
        assert rel_l2(ecg_b[i], ecg) <= ECG_TOL
        assert np.allclose(crit_b[i], crit, rtol=0, atol=1e-4)
        assert viol_b[i] == viol


def test_eval_128_twelve_leads(engine, tmp_path):
    from ekgsim_gb300.engine import Heart
    w, c = _workload(tmp_path, 1)
    s = O.load_setup(str(tmp_path))
    h = Heart.from_ini(engine, os.path.join(str(tmp_path), "simulator.ini"))
    g = synth.genes_for(c["spec"], 1, 1)
    crit_ref, viol_ref, ecg_ref, _, _ = O.evaluate(s, g)
    crit, viol, ecg, _, _ = h.eval(g, want_ecg=True)
    assert ecg.shape == (12, 600)
    assert rel_l2(ecg, ecg_ref) <= ECG_TOL
    assert np.allclose(crit, crit_ref, rtol=0, atol=1e-4)


def test_bad_inputs(engine, tmp_path):
    from ekgsim_gb300.engine import EkgError, Heart
    spec = synth.small_spec(16)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, [1, 2, 2])
    with pytest.raises(EkgError) as e:
        Heart.create(engine, np.abs(grid), tm, np.array([[30.0, 30, 30]]))
    assert e.value.code == -6  # no stimulus voxel
    with pytest.raises(EkgError) as e:
        Heart.create(engine, grid, tm[:3, :3], np.array([[30.0, 30, 30]]))
    assert e.value.code == -7  # conduction matrix misses layer 3
    w, c = _workload(tmp_path, 0)
    h = Heart.from_ini(engine, os.path.join(str(tmp_path), "simulator.ini"))
    with pytest.raises(EkgError):
        h.eval(np.zeros(5))
    g = synth.genes_for(c["spec"], 0, 0)
    g[3] = np.nan
    with pytest.raises(EkgError):
        h.eval(g)


def test_contract_kernels_agree(tmp_path):
    """The band-form, tensor-core and dense CUDA-core contractions give the same ECG within the
    tolerance, and each matches the FP64 oracle."""
    from ekgsim_gb300.engine import Engine, Heart
    spec = synth.config(0)["spec"]
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    lk = layer_k_for(spec, 3)
    out = {}
    for impl in ("band", "umma", "cuda"):
        os.environ["EKG_CONTRACT"] = impl
        try:
            e = Engine(0)
            h = Heart.create(e, grid, tm, leads, "3D4", 0.0, 600.0, 1.0)
            out[impl] = h.simulate(lk)
            h.close()
            e.close()
        finally:
            os.environ.pop("EKG_CONTRACT", None)
    at, layer = O.activation(grid, tm)
    ref = O.run(layer, at, lk, leads, "3D4", 0.0, 600.0, 1.0)
    for impl in ("band", "umma", "cuda"):
        assert rel_l2(out[impl], ref) <= ECG_TOL, impl
    assert rel_l2(out["umma"], out["cuda"]) <= ECG_TOL
    assert rel_l2(out["band"], out["cuda"]) <= ECG_TOL


@pytest.mark.parametrize("case", ["fine_dt", "k4_zero", "k4_negative", "sharp_k1", "slow_k1", "two_blobs"])
def test_per_simulation_zero_steady_band_cases(case):
    """The per-simulation contractions split each chunk's steps into zero, steady and band runs:
    a fine time axis (bands of 100+ steps, several passes), k4 = 0 and k4 < 0 (no zero run),
    sharp and slow upstrokes, and a heart with a second, unstimulated blob (activation time 0)."""
    from ekgsim_gb300.engine import Engine, Heart
    spec = synth.small_spec(24, n_leads=3)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    steps, dt = 300, 1.0
    lk = layer_k_for(spec, 1)
    if case == "fine_dt":
        steps, dt = 600, 0.1
    elif case == "k4_zero":
        lk[:, 4] = 0.0
    elif case == "k4_negative":
        lk[:, 4] = -0.02
    elif case == "sharp_k1":
        lk[:, 1] = 20.0
    elif case == "slow_k1":
        lk[:, 1] = 0.3
    elif case == "two_blobs":
        rng = np.random.Generator(np.random.PCG64(5))
        grid = np.zeros((20, 22, 18), dtype=np.int32)
        grid[2:9, 3:12, 2:10] = rng.integers(1, 4, size=(7, 9, 8))
        grid[12:18, 10:20, 8:16] = rng.integers(1, 4, size=(6, 10, 8))
        grid[3, 4, 3] = -abs(grid[3, 4, 3])
        leads = np.array([[60.0, 11.0, 9.0], [10.0, 60.0, 9.0], [-40.0, 5.0, 30.0]])
    at, layer = O.activation(grid, tm)
    ref = O.run(layer, at, lk, leads, "3D4", 0.0, steps * dt, dt)
    for impl in ("band", "umma"):
        os.environ["EKG_CONTRACT"] = impl
        try:
            e = Engine(0)
            h = Heart.create(e, grid, tm, leads, "3D4", 0.0, steps * dt, dt)
            ecg = h.simulate(lk)
            h.close()
            e.close()
        finally:
            os.environ.pop("EKG_CONTRACT", None)
        assert rel_l2(ecg, ref) <= ECG_TOL, impl


def test_per_simulation_twenty_leads_three_moved(engine):
    """Per-simulation form with two 16-lead blocks (the second partial) and an odd number of
    moved leads (the field kernel evaluates moved leads in pairs)."""
    spec = synth.small_spec(24, n_leads=20)
    h, grid, tm, leads = make_heart(engine, spec, steps=250)
    at, layer = O.activation(grid, tm)
    lk = layer_k_for(spec, 2)
    disp = np.zeros((20, 2))
    disp[:3] = [[3.0, -2.0], [-1.5, 4.0], [2.5, 2.5]]
    moved = O.move_leads(leads, disp)
    assert np.array_equal(moved[3:], leads[3:]) and not np.array_equal(moved[:3], leads[:3])
    ecg = h.simulate(lk, moved)
    ref = O.run(layer, at, lk, moved, "3D4", 0.0, 250.0, 1.0)
    assert ecg.shape == (20, 250)
    assert rel_l2(ecg, ref) <= ECG_TOL


def test_batch_fast_approximation_and_endo_epi_match_single(engine):
    """The fast-approximation criterion and the endo-epi criterion of a batch (computed on the host
    pool) equal those of single evaluations bit for bit; with a limit that gates every simulation,
    all criteria come from the approximation."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(24, n_leads=2)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, 200.0, 1.0)
    target = [t for t in synth.analytic_target(2, 200, 5)]
    genes = np.stack([synth.genes_for(spec, r, 0) for r in range(12)])
    for limit in (2.0, 0.05):
        h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6,
                   fast_is_criterion=True, fast_delay=10.0, fast_limit=limit, endo_epi_delay=2.0)
        assert h.eval_shape()[1] == 4  # two leads, the approximation, endo-epi
        crit_b, viol_b = h.eval_batch(genes)
        for i in range(len(genes)):
            crit1, viol1 = h.eval(genes[i])[:2]
            assert h.simulation_done() == (not crit1[2] > limit)
            assert crit_b[i][2] == crit1[2] and crit_b[i][3] == crit1[3]
            assert np.allclose(crit_b[i], crit1, rtol=0, atol=1e-4)
            assert viol_b[i] == viol1
            if limit < 2.0 and crit1[2] > limit:  # gated: every lead's criterion is the approximation's
                assert crit_b[i][0] == crit1[2] and crit_b[i][1] == crit1[2]


def _batch_vs_oracle(engine, spec, steps, genes, layer_k_fn, two_bases=False):
    from ekgsim_gb300.engine import Heart
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = synth.analytic_target(spec.n_leads, steps, 3)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target], mid_position=0.6)
    crit_b, viol_b, ecg_b = h.eval_batch(genes, want_ecg=True)
    at, layer = O.activation(grid, tm)
    worst = 0.0
    for i, g in enumerate(genes):
        lk = layer_k_fn(g)
        moved = O.move_leads(leads, g[12:12 + 2 * spec.n_leads].reshape(-1, 2))
        ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
        worst = max(worst, rel_l2(ecg_b[i], ref))
        crit1, viol1, ecg1, _, _ = h.eval(g, want_ecg=True)
        assert rel_l2(ecg_b[i], ecg1) <= ECG_TOL
        assert np.allclose(crit_b[i], crit1, rtol=0, atol=1e-4)
    return worst


def test_batched_form_matches_oracle_64(engine):
    """Separable batched form (static-lead Taylor basis + moved-lead GEMM) against the oracle."""
    c = synth.config(0)
    spec = c["spec"]
    genes = np.stack([synth.genes_for(spec, r, 0) for r in range(6)])
    worst = _batch_vs_oracle(engine, spec, 600, genes, lambda g: O.layer_aps(
        3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi", 0.6, g[:12])[0])
    assert worst <= ECG_TOL


def test_batched_form_twelve_leads_static_and_moved(engine):
    spec = synth.small_spec(40, n_leads=12)
    genes = np.stack([synth.genes_for(spec, r, 0) for r in range(5)])
    worst = _batch_vs_oracle(engine, spec, 400, genes, lambda g: O.layer_aps(
        3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi", 0.6, g[:12])[0])
    assert worst <= ECG_TOL


def test_batched_two_bases_free_k3(engine):
    """k3 free per simulation: the batched form keeps both bases (N = 128 / 32 tiles, six MMAs per K
    step) and still matches the oracle."""
    from ekgsim_gb300.engine import Heart
    spec = synth.config(0)["spec"]
    steps = 500
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    free = [3, 5, 6, 7, 8]
    target = synth.analytic_target(spec.n_leads, steps, 4)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, free, [t for t in target], mid_position=0.6)
    ng, _ = h.eval_shape()
    lo, hi = h.gene_bounds()
    rng = np.random.Generator(np.random.PCG64(11))
    genes = lo + (hi - lo) * rng.random((20, ng))
    # lead displacements as in the README-bounded vectors (the AP genes above are free within bounds)
    genes[:, 15:] = np.stack([synth.genes_for(spec, r, 0)[12:] for r in range(20)])
    _, _, ecg_b = h.eval_batch(genes, want_ecg=True)
    at, layer = O.activation(grid, tm)
    for i in (0, 7, 19):
        g = genes[i]
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, free, "endo-mid-epi", 0.6,
                         g[:15])[0]
        moved = O.move_leads(leads, g[15:15 + 2 * spec.n_leads].reshape(-1, 2))
        ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
        assert rel_l2(ecg_b[i], ref) <= ECG_TOL


def test_per_simulation_form_many_moved_rows(engine):
    """k1 free per simulation (the per-simulation form): 70 simulations with 280 moved rows (all four
    leads displaced, some to within a few cells of the heart) and 140 (two leads), 20 with 40 and 6
    with 12, which the persistent row kernel evaluates in its layouts (four rows per thread, one row
    per thread with the stage's chunks split over two and four warp groups); the band contraction
    scales the rows and the chunk reduction rebuilds the zero and steady runs.  A spread of results
    against the oracle, every result against its single evaluation (one simulation: the per-AP
    lead-field kernel)."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(40, n_leads=4, seed=37)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    free = [1, 5, 6, 7, 8]
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, free,
               [t for t in synth.analytic_target(spec.n_leads, steps, 9)], mid_position=0.6)
    ng, _ = h.eval_shape()
    lo, hi = h.gene_bounds()
    rng = np.random.Generator(np.random.PCG64(41))
    n = 70
    genes = lo + (hi - lo) * rng.random((n, ng))
    genes[:, 15:] = rng.uniform(-50.0, 50.0, size=(n, 2 * spec.n_leads))
    at, layer = O.activation(grid, tm)
    nz = np.argwhere(layer > 0).astype(float) + 1.0  # bordered voxel coordinates (z, y, x)
    for nmoved, ns in ((4, 70), (2, 70), (2, 20), (2, 6)):
        gs = genes[:ns].copy()
        gs[:, 15 + 2 * nmoved:] = 0.0
        lks = np.stack([O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, free, "endo-mid-epi",
                                    0.6, g[:15])[0] for g in gs])
        moveds = np.stack([O.move_leads(leads, g[15:].reshape(-1, 2)) for g in gs])
        assert not h.benchmark(lks, moveds, warmup=1, iters=1)["batched"]
        if ns == n:
            mind = [min(np.sqrt(((nz - p) ** 2).sum(axis=1)).min() for p in m[:nmoved]) for m in moveds]
            assert min(mind) < 20.0 and max(mind) > 21.0
        crit_b, viol_b, ecg_b = h.eval_batch(gs, want_ecg=True)
        for i in sorted({0, ns // 3, (2 * ns) // 3, ns - 1}):
            ref = O.run(layer, at, lks[i], moveds[i], "3D4", 0.0, float(steps), 1.0)
            assert rel_l2(ecg_b[i], ref) <= ECG_TOL, (nmoved, ns, i)
        for i in range(ns):
            c1, v1, e1 = h.eval_batch(gs[i:i + 1], want_ecg=True)
            assert rel_l2(ecg_b[i], e1[0]) <= ECG_TOL, (nmoved, ns, i)
            assert np.allclose(crit_b[i], c1[0], rtol=0, atol=1e-4) and viol_b[i] == v1[0]
    h.close()


def test_single_simulation_batched_form(engine):
    """Repeated single evaluations with the same k1, k4 switch to the batched form (static-lead basis +
    32-row band GEMM); the first call uses the per-simulation form.  Both match the oracle."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(40, n_leads=4, seed=21)
    steps = 400
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = synth.analytic_target(spec.n_leads, steps, 5)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target], mid_position=0.6)
    at, layer = O.activation(grid, tm)
    for r in range(3):
        g = synth.genes_for(spec, 50 + r, 0)
        crit, viol, ecg, _, _ = h.eval(g, want_ecg=True)
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi",
                         0.6, g[:12])[0]
        moved = O.move_leads(leads, g[12:12 + 2 * spec.n_leads].reshape(-1, 2))
        ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
        assert rel_l2(ecg, ref) <= ECG_TOL


def test_bsm_256_64lead_batched(engine):
    """The large body-surface-map configuration at full size: 256^3 ellipsoid, 10 layers with seeded
    delays, 64 electrodes on an ellipsoidal torso, 800 steps, a batch of 64 vectors.  Activation times
    bit-exact; one simulation of the batch against the FP64 oracle."""
    from ekgsim_gb300.engine import Heart
    c = synth.config(4)
    spec, steps, batch = c["spec"], c["steps"], c["batch"]
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    at, layer = O.activation(grid, tm)
    assert np.array_equal(h.activation().view(np.int64), at.view(np.int64))
    target = synth.analytic_target(spec.n_leads, steps, 6)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target], mid_position=0.6)
    genes = np.stack([synth.genes_for(spec, r, 4) for r in range(batch)])
    crit, viol, ecg = h.eval_batch(genes, want_ecg=True)
    assert np.isfinite(crit).all() and np.isfinite(ecg).all()
    g = genes[5]
    lk = O.layer_aps(spec.n_layers, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                     "endo-mid-epi", 0.6, g[:12])[0]
    moved = O.move_leads(leads, g[12:12 + 2 * spec.n_leads].reshape(-1, 2))
    ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
    assert rel_l2(ecg[5], ref) <= ECG_TOL
    h.close()


def _batched_general(engine, spec, nhood, start, length, dt, n, seed=9):
    """Batched evaluation (eval_batch) with any neighbourhood and time axis against the oracle."""
    from ekgsim_gb300.engine import Heart
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, nhood, start, length, dt)
    steps = h.steps
    target = synth.analytic_target(spec.n_leads, steps, seed)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target], mid_position=0.6)
    genes = np.stack([synth.genes_for(spec, 60 + r, 0) for r in range(n)])
    _, _, ecg_b = h.eval_batch(genes, want_ecg=True)
    at, layer = O.activation(grid, tm)
    worst = 0.0
    for i in (0, n - 1):
        g = genes[i]
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi",
                         0.6, g[:12])[0]
        moved = O.move_leads(leads, g[12:12 + 2 * spec.n_leads].reshape(-1, 2))
        ref = O.run(layer, at, lk, moved, nhood, start, length, dt)
        worst = max(worst, rel_l2(ecg_b[i], ref))
    h.close()
    return worst


@pytest.mark.parametrize("nhood", ["cube", "2D8", "2D4"])
def test_batched_form_neighbourhoods(engine, nhood):
    """Batched form with the general-neighbourhood operand kernel (the 26-neighbour cube also takes
    the closed-form interior field; the 2-D sets have no cube symmetry and keep the exact sum)."""
    assert _batched_general(engine, synth.small_spec(24, n_leads=3), nhood, 0.0, 250.0, 1.0, 5) <= ECG_TOL


def test_batched_form_fine_time_axis(engine):
    """dt = 1/32 ms over 100 ms (3200 steps): tiles of 4 ms, bands spanning several tiles and more
    tiles before the first all-steady one than steady-prefix entries, so tiles share entries."""
    assert _batched_general(engine, synth.small_spec(32, n_leads=2), "3D4", 2.0, 100.0, 0.03125, 4) <= ECG_TOL


def test_graph_replay_is_bit_identical():
    """Repeated passes replay a captured CUDA graph (from the third pass with the same shape); the
    results are bitwise those of direct launches (EKG_GRAPHS=0), single and batched."""
    from ekgsim_gb300.engine import Engine, Heart
    spec = synth.small_spec(32, n_leads=3, seed=13)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    target = synth.analytic_target(spec.n_leads, 300, 8)
    genes = np.stack([synth.genes_for(spec, r, 0) for r in range(6)])
    out = {}
    for flag in ("1", "0"):
        os.environ["EKG_GRAPHS"] = flag
        try:
            e = Engine(0)
            h = Heart.create(e, grid, tm, leads, "3D4", 0.0, 300.0, 1.0)
            h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target],
                       mid_position=0.6)
            res = []
            for _ in range(4):
                res.append(h.eval_batch(genes, want_ecg=True))
                res.append(h.eval(genes[2], want_ecg=True)[:3])
            out[flag] = res
            h.close()
            e.close()
        finally:
            os.environ.pop("EKG_GRAPHS", None)
    for a, b in zip(out["1"], out["0"]):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_criteria_modes_match_fp64_compare(engine, mode):
    """Every comparison mode (1 RMS, 2 Pearson, 3 devFromLinear, 4 vector correlation) gives the
    FP64 comparison of the engine's own ECG with the target (the oracle's compare, vectorMath.h),
    for a batch of 256 (one warp per simulation and lead) and a single evaluation (four warps);
    the target is shorter than the simulation, so the compared length is the target's."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(40, n_leads=4, seed=5)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = synth.analytic_target(spec.n_leads, steps - 20, 9)
    offs = [0.5, 1.0, 0.25, 2.0]
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target],
               target_offsets=offs, mid_position=0.6, comparison_mode=mode)
    genes = np.stack([synth.genes_for(spec, r, 0) for r in range(256)])
    crit_b, _, ecg_b = h.eval_batch(genes, want_ecg=True)
    crit_1, _, ecg_1, _, _ = h.eval(genes[3], want_ecg=True)
    for crit, ecg in [(crit_b[0], ecg_b[0]), (crit_b[100], ecg_b[100]), (crit_b[255], ecg_b[255]), (crit_1, ecg_1)]:
        for l in range(spec.n_leads):
            ref = O.clamp(O.compare(mode, ecg[l], target[l], offs[l]))
            assert crit[l] == pytest.approx(ref, rel=1e-9, abs=1e-12), (mode, l)


def test_batched_form_plane_fronts_large_aps(engine):
    """A slab stimulated on a whole plane activates plane by plane, so every AP holds a full plane
    of voxels and a 32-AP stage holds thousands: the operand kernel reads those stages' voxel
    records from global memory instead of its shared-memory copy.  Batched ECGs (more than 16
    simulations, the persistent operand kernel) match the oracle."""
    from ekgsim_gb300.engine import Heart
    n, steps, nl = 24, 300, 3
    grid = np.zeros((n, n, n), dtype=np.int16)
    for z in range(4, 22):
        grid[z, 3:21, 3:21] = 1 + min(2, (z - 4) // 6)
    grid[4, 3:21, 3:21] = -1
    tm = synth.transfer_matrix(nl, [1, 2, 2])
    rng = np.random.Generator(np.random.PCG64(17))
    v = rng.normal(size=(4, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    leads = (n / 2.0 + 40.0 * v)[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = synth.analytic_target(4, steps, 5)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target], mid_position=0.6)
    spec = synth.small_spec(40, n_leads=4, seed=5)
    genes = np.stack([synth.genes_for(spec, r, 0) for r in range(20)])
    _, _, ecg_b = h.eval_batch(genes, want_ecg=True)
    at, layer = O.activation(grid, tm)
    for i in (0, 9, 19):
        g = genes[i]
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi",
                         0.6, g[:12])[0]
        moved = O.move_leads(leads, g[12:12 + 8].reshape(-1, 2))
        ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
        assert rel_l2(ecg_b[i], ref) <= ECG_TOL


def test_queued_batches_match_synchronous(engine):
    """Queued batched evaluations (two in flight, a third submission completing the oldest) give the
    same criteria, violations and ECGs as synchronous calls, bit for bit."""
    from ekgsim_gb300 import engine as E
    spec = synth.small_spec(40, n_leads=4, seed=8)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = E.Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = synth.analytic_target(spec.n_leads, steps, 2)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], [t for t in target], mid_position=0.6)
    batches = [np.stack([synth.genes_for(spec, 40 * b + r, 0) for r in range(20 + 3 * b)]) for b in range(3)]
    ref = [h.eval_batch(g, want_ecg=True) for g in batches]
    outs = [(np.empty_like(r[0]), np.empty_like(r[1]), np.empty_like(r[2])) for r in ref]
    for o in outs:
        for a in o:
            E.host_register(a)
    try:
        t0 = h.eval_batch_submit(batches[0], outs[0], want_ecg=True)
        t1 = h.eval_batch_submit(batches[1], outs[1], want_ecg=True)
        t2 = h.eval_batch_submit(batches[2], outs[2], want_ecg=True)  # completes the first
        h.eval_batch_wait(t2)
        h.eval_batch_wait(t0)
        h.eval_batch_wait(t1)
        for o, r in zip(outs, ref):
            for a, b in zip(o, r):
                assert np.array_equal(a, b)
    finally:
        for o in outs:
            for a in o:
                E.host_unregister(a)


def test_c3_batched_full_size(engine):
    """The batched configuration at full size: 160^3 ellipsoid (wall 14, 3 layers), 12 leads, 600
    steps, 256 distinct seeded vectors in one batched evaluation.  Activation times bitwise at
    160^3; 8 results spread over the batch (first, last, middle, seeded random) against the FP64
    oracle; every result against the per-simulation form of a second engine (batched form off)."""
    from ekgsim_gb300.engine import Engine, Heart
    c = synth.config(2)
    spec, steps, batch = c["spec"], c["steps"], c["batch"]
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    target = [t for t in synth.analytic_target(spec.n_leads, steps, spec.seed + 999)]
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    at, layer = O.activation(grid, tm)
    assert np.array_equal(h.activation().view(np.int64), at.view(np.int64))
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6)
    genes = np.stack([synth.genes_for(spec, r, 2) for r in range(batch)])
    assert len({g.tobytes() for g in genes}) == batch
    crit_b, viol_b, ecg_b = h.eval_batch(genes, want_ecg=True)
    assert np.isfinite(ecg_b).all()
    pick = sorted({0, batch // 2, batch - 1} | set(int(x) for x in np.random.Generator(np.random.PCG64(31)).choice(
        np.arange(1, batch - 1), size=5, replace=False)))
    assert len(pick) >= 8
    for i in pick:
        g = genes[i]
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi",
                         0.6, g[:12])[0]
        moved = O.move_leads(leads, g[12:].reshape(-1, 2))
        ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
        assert rel_l2(ecg_b[i], ref) <= ECG_TOL, i
        for l in range(spec.n_leads):
            assert crit_b[i][l] == pytest.approx(O.clamp(O.compare(2, ref[l], target[l])), abs=1e-4)
    h.close()
    os.environ["EKG_BATCHED"] = "0"
    try:
        e2 = Engine(0)
    finally:
        os.environ.pop("EKG_BATCHED", None)
    h2 = Heart.create(e2, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    h2.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6)
    crit_p, viol_p, ecg_p = h2.eval_batch(genes, want_ecg=True)
    for i in range(batch):
        assert rel_l2(ecg_b[i], ecg_p[i]) <= ECG_TOL, i
    assert np.allclose(crit_b, crit_p, rtol=0, atol=1e-4)
    assert np.array_equal(viol_b, viol_p)
    h2.close()
    e2.close()


def test_bounded_wait_runs_out_and_device_stays_usable(engine):
    """Failure detection without a GPU fault: a kernel waits on an mbarrier that nothing arrives on,
    with the contraction kernels' bounded wait and a short poll limit; it records the timeout in
    the error word, releases its tensor memory and returns, the call reports EKG_ERR_TIMEOUT, and
    the device keeps working (a heart is created and simulated afterwards)."""
    from ekgsim_gb300 import _lib as L
    from ekgsim_gb300.engine import Heart
    lib = L.load()
    assert lib.ekg_selftest_bounded_wait(0, 1 << 12) == -5
    assert "bounded device wait ran out" in lib.ekg_last_error().decode()
    assert lib.ekg_selftest_bounded_wait(0, 0) == -1
    spec = synth.small_spec(16)
    h, grid, tm, leads = make_heart(engine, spec, steps=50)
    at, layer = O.activation(grid, tm)
    assert np.array_equal(h.activation().view(np.int64), at.view(np.int64))
    lk = layer_k_for(spec)
    assert rel_l2(h.simulate(lk), O.run(layer, at, lk, leads, "3D4", 0.0, 50.0, 1.0)) <= ECG_TOL


def test_activation_round_cap_reports_not_converged():
    """The activation-time relaxation gives up after its round cap with EKG_ERR_CA_NOT_CONVERGED
    (the cap set low through EKG_CA_ROUND_CAP); an engine with the default cap converges on the same
    heart, bit-exact against the oracle."""
    from ekgsim_gb300.engine import EkgError, Engine, Heart
    spec = synth.small_spec(40)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    os.environ["EKG_CA_ROUND_CAP"] = "2"
    try:
        e = Engine(0)
    finally:
        os.environ.pop("EKG_CA_ROUND_CAP", None)
    with pytest.raises(EkgError) as err:
        Heart.create(e, grid, tm, np.array([[60.0, 60.0, 60.0]]), "3D4", 0.0, 10.0, 1.0)
    assert err.value.code == -3
    e.close()
    e2 = Engine(0)
    h = Heart.create(e2, grid, tm, np.array([[60.0, 60.0, 60.0]]), "3D4", 0.0, 10.0, 1.0)
    assert h.info.ca_rounds > 2
    at, _ = O.activation(grid, tm)
    assert np.array_equal(h.activation().view(np.int64), at.view(np.int64))
    h.close()
    e2.close()


def test_autotuned_shape_keeps_parity(tmp_path):
    """The autotuner times every candidate launch shape on the real heart and keeps the fastest;
    batched results with the tuned shape match the FP64 oracle and the built-in shape's results
    within the tolerance, the choice is written to the cache file, and a new engine reads it back
    for the same pass shape (its results equal the tuned engine's bit for bit)."""
    from ekgsim_gb300.engine import Engine, Heart
    spec = synth.small_spec(48, n_leads=6, seed=23)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    target = [t for t in synth.analytic_target(spec.n_leads, steps, 4)]
    genes = np.stack([synth.genes_for(spec, 70 + r, 0) for r in range(96)])
    cache = str(tmp_path / "tune.txt")
    out = {}
    for tag in ("builtin", "tuned", "cached"):
        if tag != "builtin":
            os.environ["EKG_TUNE_CACHE"] = cache
        try:
            e = Engine(0)
        finally:
            os.environ.pop("EKG_TUNE_CACHE", None)
        h = Heart.create(e, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
        h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6)
        if tag == "tuned":
            lk = np.stack([O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                                       "endo-mid-epi", 0.6, g[:12])[0] for g in genes])
            moved = np.stack([O.move_leads(leads, g[12:].reshape(-1, 2)) for g in genes])
            t = h.tune(lk, moved, reps=2)
            assert t["candidates"] >= 3 and t["tile_rows"] in (32, 128, 256) and t["ms"] > 0
            assert t["ms"] <= t["builtin_ms"] * 1.0001
            assert os.path.exists(cache)
        out[tag] = h.eval_batch(genes, want_ecg=True)
        h.close()
        e.close()
    at, layer = O.activation(grid, tm)
    for i in (0, 50, 95):
        g = genes[i]
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi",
                         0.6, g[:12])[0]
        ref = O.run(layer, at, lk, O.move_leads(leads, g[12:].reshape(-1, 2)), "3D4", 0.0, float(steps), 1.0)
        assert rel_l2(out["tuned"][2][i], ref) <= ECG_TOL
        assert rel_l2(out["tuned"][2][i], out["builtin"][2][i]) <= ECG_TOL
    assert np.allclose(out["tuned"][0], out["builtin"][0], rtol=0, atol=1e-4)
    for a, b in zip(out["tuned"], out["cached"]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("n", [16, 40, 128])
def test_activation_tile_rounds_and_buckets_agree(n):
    """The two relaxations -- time buckets (default where the lags allow) and tile rounds
    (EKG_CA=tiles, and the fallback) -- give the oracle's activation times bit for bit."""
    from ekgsim_gb300.engine import Engine, Heart
    spec = synth.small_spec(n) if n < 128 else synth.config(1)["spec"]
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(spec.n_layers, spec.delays)
    at_ref, _ = O.activation(grid, tm)
    for mode in ("tiles", "buckets"):
        if mode == "tiles":
            os.environ["EKG_CA"] = "tiles"
        try:
            e = Engine(0)
        finally:
            os.environ.pop("EKG_CA", None)
        h = Heart.create(e, grid, tm, np.array([[n * 2.0, n * 2.0, n * 2.0]]), "3D4", 0.0, 10.0, 1.0)
        assert np.array_equal(h.activation().view(np.int64), at_ref.view(np.int64)), mode
        h.close()
        e.close()


@pytest.mark.parametrize("case", ["single_voxel", "ragged", "plane", "zero_lag", "isolated_stimulus"])
def test_activation_edge_shapes(case):
    """Activation times bit-exact against the oracle on edge shapes, with both relaxations: a
    one-voxel heart, extents that are not multiples of the 8-cell tiles, a one-cell-thick plane, a
    conduction matrix with a zero delay (no time buckets: the tile rounds run), and a stimulus voxel
    without non-empty neighbours next to an unreachable block; the ECG of the ragged heart too."""
    from ekgsim_gb300.engine import Engine, Heart
    rng = np.random.Generator(np.random.PCG64(41))
    tm = synth.transfer_matrix(3, [1, 2, 2])
    if case == "single_voxel":
        grid = np.array([[[-1]]], dtype=np.int32)
    elif case == "ragged":
        grid = rng.integers(0, 4, size=(13, 17, 11)).astype(np.int32)
        grid[6, 8, 5] = -2
    elif case == "plane":
        grid = rng.integers(1, 4, size=(1, 37, 29)).astype(np.int32)
        grid[0, 3, 4] = -1
    elif case == "zero_lag":
        grid = rng.integers(1, 4, size=(12, 10, 14)).astype(np.int32)
        grid[0, 0, 0] = -1
        tm = tm.copy()
        tm[2, 3] = 0.0
    else:
        grid = np.zeros((10, 10, 10), dtype=np.int32)
        grid[1, 1, 1] = -1
        grid[5:9, 5:9, 5:9] = 2
    at_ref, layer = O.activation(grid, tm)
    leads = np.array([[30.0, 25.0, 20.0], [-12.0, 4.0, 33.0]])
    for mode in ("buckets", "tiles"):
        if mode == "tiles":
            os.environ["EKG_CA"] = "tiles"
        try:
            e = Engine(0)
        finally:
            os.environ.pop("EKG_CA", None)
        h = Heart.create(e, grid, tm, leads, "3D4", 0.0, 60.0, 1.0)
        assert np.array_equal(h.activation().view(np.int64), at_ref.view(np.int64)), mode
        if case == "zero_lag":
            assert h.info.ca_buckets == 0
        if case == "ragged":
            lk = layer_k_for(synth.small_spec(16), 3)
            assert rel_l2(h.simulate(lk), O.run(layer, at_ref, lk, leads, "3D4", 0.0, 60.0, 1.0)) <= ECG_TOL
        h.close()
        e.close()


def test_batched_form_resting_potential(engine):
    """The resting potential k0 leaves sum_L k0_L sum_{a in L} W[l, a] on every sample.  With k0 the
    same in every layer (-86 mV) it cancels in the dipoles (sum_a W[l, a] = 0); with k0 differing
    between layers the batched form adds it, for the static leads (layer sums of the resident lead
    field) and for the moved ones (per-part field sums written by the operand kernel).  Both batches
    take the batched form and match the oracle and single evaluations, with two of four leads moved
    (the static and moved terms, on two streams) and with all four moved (one stream)."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(40, n_leads=4, seed=29)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = [t for t in synth.analytic_target(spec.n_leads, steps, 6)]
    at, layer = O.activation(grid, tm)
    genes = np.stack([synth.genes_for(spec, 80 + r, 0) for r in range(12)])
    genes_all = genes.copy()
    genes_all[:, 16:] = np.random.Generator(np.random.PCG64(83)).uniform(-30.0, 30.0, size=(12, 4))
    for k0s in ((-86.0, -86.0, -86.0), (-86.0, -80.0, -90.0)):
        base = [[k0] + list(synth.BASE_AP[1:]) for k0 in k0s]
        kmin, kmax = list(synth.K_MIN), list(synth.K_MAX)
        kmin[0], kmax[0] = min(k0s), max(k0s)
        h.set_eval(base, kmin, kmax, [5, 6, 7, 8], target, mid_position=0.6)
        for gs in (genes, genes_all):
            crit_b, viol_b, ecg_b = h.eval_batch(gs, want_ecg=True)
            lks = np.stack([O.layer_aps(3, np.array(base), np.array(kmin), np.array(kmax), [5, 6, 7, 8],
                                        "endo-mid-epi", 0.6, g[:12])[0] for g in gs])
            moveds = np.stack([O.move_leads(leads, g[12:].reshape(-1, 2)) for g in gs])
            assert h.benchmark(lks, moveds, warmup=1, iters=1)["batched"]
            for i in (0, 11):
                g = gs[i]
                lk = lks[i]
                # the mid layer takes the last base AP's k0 (sim.cpp:856), so the layers get -86, -90, -90
                assert (len(set(lk[:, 0])) == 1) == (len(set(k0s)) == 1)
                ref = O.run(layer, at, lk, moveds[i], "3D4", 0.0, float(steps), 1.0)
                assert rel_l2(ecg_b[i], ref) <= ECG_TOL, (k0s, i)
            # every simulation against its single evaluation
            for i in range(len(gs)):
                c1, v1, e1 = h.eval_batch(gs[i:i + 1], want_ecg=True)
                assert rel_l2(ecg_b[i], e1[0]) <= ECG_TOL, (k0s, i)
                assert np.allclose(crit_b[i], c1[0], rtol=0, atol=1e-4) and viol_b[i] == v1[0]
    h.close()


def test_batched_operand_layouts(engine):
    """The batched form's operand kernel picks its layout from the moved rows: the per-(AP, simulation)
    kernel up to 4 simulations, one row per thread with a stage's chunks split over four, two or one
    warp groups up to 128 rows, four rows per thread split over two groups up to 256, unsplit above.
    The same gene vectors in batches of 3, 5, 30, 64, 100 and 130 simulations (2 moved leads) give
    the same ECGs within the tolerance, and a spread of them matches the oracle."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(40, n_leads=4, seed=43)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
               [t for t in synth.analytic_target(spec.n_leads, steps, 5)], mid_position=0.6)
    genes = np.stack([synth.genes_for(spec, 500 + r, 0) for r in range(130)])
    at, layer = O.activation(grid, tm)
    first = None
    for n in (3, 5, 30, 64, 100, 130):
        lks = np.stack([O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                                    "endo-mid-epi", 0.6, g[:12])[0] for g in genes[:n]])
        moveds = np.stack([O.move_leads(leads, g[12:].reshape(-1, 2)) for g in genes[:n]])
        assert h.benchmark(lks, moveds, warmup=1, iters=1)["batched"]
        crit, viol, ecg = h.eval_batch(genes[:n], want_ecg=True)
        if first is None:
            first = ecg[:3].copy()
        for i in range(3):
            assert rel_l2(ecg[i], first[i]) <= ECG_TOL, (n, i)
        for i in sorted({0, n // 2, n - 1}):
            ref = O.run(layer, at, lks[i], moveds[i], "3D4", 0.0, float(steps), 1.0)
            assert rel_l2(ecg[i], ref) <= ECG_TOL, (n, i)
    h.close()


def test_cube_neighbourhood_moved_leads(engine):
    """The general-neighbourhood instances of the moved-lead field kernels ("cube": 26 neighbours,
    with its own closed-form interior coefficients): the batched form at 30 and 130 simulations
    (one row per thread, four rows per thread) and the per-simulation form with k1 free at 20
    simulations (the row kernel), against the oracle and against single evaluations."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(32, n_leads=3, seed=47)
    steps = 250
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "cube", 0.0, float(steps), 1.0)
    target = [t for t in synth.analytic_target(spec.n_leads, steps, 3)]
    at, layer = O.activation(grid, tm)
    # batched form (k1, k4 shared)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6)
    genes = np.stack([synth.genes_for(spec, 700 + r, 0) for r in range(130)])
    first = None
    for n in (30, 130):
        lks = np.stack([O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                                    "endo-mid-epi", 0.6, g[:12])[0] for g in genes[:n]])
        moveds = np.stack([O.move_leads(leads, g[12:].reshape(-1, 2)) for g in genes[:n]])
        assert h.benchmark(lks, moveds, warmup=1, iters=1)["batched"]
        _, _, ecg = h.eval_batch(genes[:n], want_ecg=True)
        if first is None:
            first = ecg[:3].copy()
        for i in range(3):
            assert rel_l2(ecg[i], first[i]) <= ECG_TOL, (n, i)
        for i in sorted({0, n // 2, n - 1}):
            ref = O.run(layer, at, lks[i], moveds[i], "cube", 0.0, float(steps), 1.0)
            assert rel_l2(ecg[i], ref) <= ECG_TOL, (n, i)
    # per-simulation form (k1 free)
    free = [1, 5, 6, 7, 8]
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, free, target, mid_position=0.6)
    ng, _ = h.eval_shape()
    lo, hi = h.gene_bounds()
    rng = np.random.Generator(np.random.PCG64(53))
    g2 = lo + (hi - lo) * rng.random((20, ng))
    g2[:, 15:] = np.stack([synth.genes_for(spec, 800 + r, 0)[12:] for r in range(20)])
    lks = np.stack([O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, free, "endo-mid-epi",
                                0.6, g[:15])[0] for g in g2])
    moveds = np.stack([O.move_leads(leads, g[15:].reshape(-1, 2)) for g in g2])
    assert not h.benchmark(lks, moveds, warmup=1, iters=1)["batched"]
    crit_b, viol_b, ecg_b = h.eval_batch(g2, want_ecg=True)
    for i in (0, 10, 19):
        ref = O.run(layer, at, lks[i], moveds[i], "cube", 0.0, float(steps), 1.0)
        assert rel_l2(ecg_b[i], ref) <= ECG_TOL, i
    for i in range(20):
        c1, v1, e1 = h.eval_batch(g2[i:i + 1], want_ecg=True)
        assert rel_l2(ecg_b[i], e1[0]) <= ECG_TOL, i
    h.close()


def test_batched_all_leads_moved_and_near_heart(engine):
    """Every lead carries displacement genes (the reference's usual "optimize measuring points"
    case, 12 + 2L genes), some of them moving leads to within a few cells of the heart, so that the
    operand kernel takes both its closed-form path (stages far from every lead of a warp) and the
    per-voxel exact path; a batch of 40 against the oracle."""
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(48, n_leads=6, seed=33)
    steps = 300
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
    target = [t for t in synth.analytic_target(spec.n_leads, steps, 7)]
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6)
    rng = np.random.Generator(np.random.PCG64(71))
    genes = np.stack([synth.genes_for(spec, 300 + r, 0) for r in range(40)])
    genes[:, 12:] = rng.uniform(-50.0, 50.0, size=(40, 2 * spec.n_leads))
    at, layer = O.activation(grid, tm)
    nz = np.argwhere(layer > 0).astype(float) + 1.0  # bordered voxel coordinates (z, y, x)
    mind = []
    for g in genes:
        moved = O.move_leads(leads, g[12:].reshape(-1, 2))
        mind.append(min(np.sqrt(((nz - p) ** 2).sum(axis=1)).min() for p in moved))
    assert min(mind) < 20.0 and max(mind) > 21.0  # both operand-kernel paths are taken
    _, _, ecg_b = h.eval_batch(genes, want_ecg=True)
    for i in (0, int(np.argmin(mind)), int(np.argmax(mind)), 39):
        g = genes[i]
        lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi",
                         0.6, g[:12])[0]
        ref = O.run(layer, at, lk, O.move_leads(leads, g[12:].reshape(-1, 2)), "3D4", 0.0, float(steps), 1.0)
        assert rel_l2(ecg_b[i], ref) <= ECG_TOL, i
    h.close()


def test_c2_batched_twelve_leads(engine, tmp_path):
    """The single-simulation configuration's heart (128^3, 12 leads, 600 steps) in the batched form:
    a batch of 16 distinct vectors, 4 of them against the oracle."""
    from ekgsim_gb300.engine import Heart
    w, c = _workload(tmp_path, 1)
    s = O.load_setup(str(tmp_path))
    h = Heart.from_ini(engine, os.path.join(str(tmp_path), "simulator.ini"))
    genes = np.stack([synth.genes_for(c["spec"], 20 + r, 1) for r in range(16)])
    crit_b, viol_b, ecg_b = h.eval_batch(genes, want_ecg=True)
    for i in (0, 5, 10, 15):
        crit_ref, viol_ref, ecg_ref, _, _ = O.evaluate(s, genes[i])
        assert rel_l2(ecg_b[i], ecg_ref) <= ECG_TOL, i
        assert np.allclose(crit_b[i], crit_ref, rtol=0, atol=1e-4)
        assert viol_b[i] == viol_ref
    h.close()
