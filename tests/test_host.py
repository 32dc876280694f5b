"""Host-side checks that need no GPU: the C ABI library loads and exports every declared entry
point; the host parts of an evaluation (gene -> layer APs, lead displacement) match the oracle bit
for bit; the oracle's own forms agree; the synthetic workload generator reproduces the sizes and
file formats it documents; the replica timing helper of the benchmark works across two ranks."""
import ctypes
import os
import re

import numpy as np
import pytest

from ekgsim_gb300 import synth
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^(?:int|double|const char \*)\s*(ekg_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from ekgsim_gb300 import _lib as L
    lib = L.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SIGNATURES, n


def test_no_device_is_an_error_not_a_crash():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from ekgsim_gb300 import _lib as L
    lib = L.load()
    h = ctypes.c_void_p()
    assert lib.ekg_engine_create(0, ctypes.byref(h)) < 0
    assert lib.ekg_last_error()


@pytest.mark.parametrize("nl,interp", [(3, "endo-mid-epi"), (4, "endo-mid-epi"), (10, "endo-mid-epi"),
                                       (24, "endo-mid-epi"), (2, "endo-epi"), (6, "endo-epi")])
def test_gene_mapping_matches_oracle(nl, interp):
    from ekgsim_gb300 import engine as E
    nb = 3 if interp == "endo-mid-epi" else 2
    base = [synth.BASE_AP] * nb
    if nb == 3:  # distinct base APs so that interpolation has work to do
        base = [synth.BASE_AP, [0, 2.4, 100, 0.88, 0.1, 0.0008, 0.08, 0.07, 280], [0, 2.6, 100, 0.92, 0.1, 0.0006,
                                                                                   0.05, 0.04, 310]]
    cfg = E.eval_config(base, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], interpolation=interp, mid_position=0.6)
    for r in range(3):
        g = synth.genes_for(synth.config(0)["spec"], r, 7)[: 4 * nb]
        lk, v = E.layer_aps(cfg, nl, g)
        lk2, v2, over = O.layer_aps(nl, np.array(base), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], interp, 0.6, g)
        assert over == 0
        assert np.array_equal(lk, lk2)
        assert v == v2


def test_violation_counts_out_of_bound_genes():
    from ekgsim_gb300 import engine as E
    cfg = E.eval_config([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], mid_position=0.6)
    g = np.array([0.0002, 0.05, 0.05, 250.0] * 3)  # k5 below its minimum by 1e-4 in every set
    _, v = E.layer_aps(cfg, 3, g)
    _, v2, _ = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                           "endo-mid-epi", 0.6, g)
    assert v == v2 and abs(v - 3e-4) < 1e-12


def test_lead_displacement_matches_oracle():
    from ekgsim_gb300 import engine as E
    rng = np.random.Generator(np.random.PCG64(3))
    pts = rng.uniform(-100, 200, size=(12, 3))
    pts[0] = [0.0, 0.0, 0.0]  # degenerate basis (normalise a zero vector)
    pts[1] = [0.0, 0.0, 5.0]
    disp = rng.uniform(-50, 50, size=(12, 2))
    assert np.array_equal(E.move_leads(pts, disp), O.move_leads(pts, disp))
    assert np.array_equal(E.move_leads(pts, None), pts)


@pytest.mark.parametrize("nhood", ["3D4", "cube", "2D4", "2D8"])
def test_oracle_forms_agree(nhood):
    """The table form of the oracle equals its reference-cost form (per-voxel AP evaluation)."""
    spec = synth.small_spec(20, n_leads=3)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    at, layer = O.activation(grid, tm)
    lk = np.tile(np.array(synth.BASE_AP), (3, 1))
    lk[:, 5:9] = [[0.0005, 0.05, 0.04, 280], [0.0007, 0.02, 0.06, 300], [0.0004, 0.08, 0.03, 260]]
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(1)))[:, ::-1].copy()
    a = O.run(layer, at, lk, leads, nhood, 0.0, 120.0, 1.0)
    b = O.run_naive(layer, at, lk, leads, nhood, 0.0, 120.0, 1.0)
    assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_oracle_activation_properties():
    """Start voxels get 1.0, empty cells 0, unreachable non-empty cells 0, and every reached
    voxel's time is the minimum over its neighbours of time + lag (the Dijkstra fixed point)."""
    g = np.zeros((9, 10, 11), dtype=np.int32)
    g[1:5, 1:6, 1:7] = 2
    g[1:3, 1:3, 1:3] = 1
    g[2, 2, 2] = -1
    g[7:9, 7:9, 8:10] = 3  # separate blob, never reached
    tm = synth.transfer_matrix(3, [1.0, 2.0, 0.5])
    at, layer = O.activation(g, tm)
    assert at[2, 2, 2] == 1.0
    assert (at[g == 0] == 0).all()
    assert (at[7:9, 7:9, 8:10] == 0).all()
    for z, y, x in zip(*np.nonzero((layer > 0) & (at > 1))):
        best = np.inf
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    z2, y2, x2 = z + dz, y + dy, x + dx
                    if (dz or dy or dx) and 0 <= z2 < 9 and 0 <= y2 < 10 and 0 <= x2 < 11 and layer[z2, y2, x2] > 0 \
                            and at[z2, y2, x2] > 0:
                        lag = tm[layer[z2, y2, x2], layer[z, y, x]] * np.sqrt(dz * dz + dy * dy + dx * dx)
                        best = min(best, at[z2, y2, x2] + lag)
        assert at[z, y, x] == best


def test_oracle_errors():
    g = np.ones((3, 3, 3), dtype=np.int32)
    with pytest.raises(RuntimeError, match="starting point"):
        O.activation(g, synth.transfer_matrix(1, [1]))
    g[1, 1, 1] = -1
    g[0, 0, 0] = 5
    with pytest.raises(RuntimeError, match="does not define layer"):
        O.activation(g, np.ones((3, 3)))


def test_synthetic_sizes_and_files(tmp_path):
    # voxel counts of the five configurations' hearts
    assert (synth.ellipsoid_heart(synth.config(0)["spec"]) != 0).sum() == 44512
    assert (synth.ellipsoid_heart(synth.config(1)["spec"]) != 0).sum() == 357272
    assert [(synth.ellipsoid_heart(h) != 0).sum() for h in synth.config(3)["hearts"][:2]] == [18864, 150664]
    spec = synth.small_spec(24, n_leads=3)
    w = synth.make_workload(str(tmp_path), spec, 50)
    grid = O.read_matrix(str(tmp_path / "model.matrix"))
    assert np.array_equal(grid.astype(np.int32), synth.ellipsoid_heart(spec))
    assert (grid < 0).sum() == spec.n_stim
    tm = O.read_matrix(str(tmp_path / "conduction.matrix"))
    assert tm.shape[0] >= 12 and tm[1, 2] == spec.delays[1]
    pts = O.read_points(str(tmp_path / "leads.txt"))
    assert np.allclose(pts[:, ::-1], w.leads_xyz)
    ini = O.read_ini(str(tmp_path / "simulator.ini"))
    assert ini["simulation"]["neighbourhood type"] == "3D4"
    g = synth.genes_for(synth.config(1)["spec"], 5, 1)
    assert g.size == 12 + 2 * 12 and (g[16:] == 0).all()
    assert (g[:16] >= synth.GENE_MIN).all() and (g[:16] <= synth.GENE_MAX).all()


def _dist_worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    v = d.max(float(rank + 1) * 1.5)
    q.put((rank, v))
    d.close()


def test_replica_timing_max_over_two_gloo_ranks():
    pytest.importorskip("torch")
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_dist_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    out = sorted(q.get(timeout=10) for _ in range(2))
    assert out == [(0, 3.0), (1, 3.0)]


def test_band_form_run_bounds():
    """The per-simulation band-form contraction replaces H_a(t) = sigma(k1 tau)((1-k3) e^{-k4 tau} + k3)
    by 0 where k1' (amin - t) >= 30.5 and (k1' - k4')(amin - t) >= 30.5, and by its sigma = 1 form
    where k1' (t - amax) >= 26.5 (k' = k log2 e).  In FP64 over the gene ranges, the dropped part
    stays below 2^-30 of the AP's amplitude before the upstroke, and FP32 rounds the sigmoid to
    exactly 1 after it."""
    l2e = 1.4426950408889634
    rng = np.random.Generator(np.random.PCG64(3))
    k1 = rng.uniform(0.3, 20.0, 2000)
    k4 = rng.uniform(0.0, 0.2, 2000) * np.minimum(1.0, k1 / 0.4)
    k3 = rng.uniform(0.0, 1.0, 2000)
    c1, c4 = k1 * l2e, k4 * l2e
    ok = c1 > c4
    # the first tau before the upstroke that the zero run covers, and a long way past it
    tz = -np.maximum(30.5 / c1, 30.5 / np.where(ok, c1 - c4, np.inf))
    for f in (1.0, 1.5, 4.0):
        tau = tz * f
        h = (1.0 - k3) * np.exp(-k4 * tau) + k3
        sig = 1.0 / (1.0 + np.exp(-k1 * tau))
        assert np.all((sig * h)[ok] <= 2.0 ** -30 * (1.0 + 1e-9))
    # the first tau after the upstroke of the steady run: 1 + 2^-x rounds to 1 in FP32
    ts = 26.5 / c1
    e1 = np.exp2(-(c1 * ts)).astype(np.float32)
    assert np.all(np.float32(1.0) + e1 == np.float32(1.0))


def test_oracle_naive_time_ranges_equal_whole_axis():
    """The reference arm of the benchmark times the reference's per-voxel loop in slices of the time
    axis; the slices give the same values as one pass over the whole axis (time advanced by += dt)."""
    spec = synth.small_spec(16, n_leads=2)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    at, layer = O.activation(grid, tm)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
    lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], "endo-mid-epi", 0.6,
                     synth.genes_for(spec, 0, 0)[:12])[0]
    full = O.run_naive(layer, at, lk, leads, "3D4", 3.0, 80.0, 0.25)
    parts = [O.run_naive_range(layer, at, lk, leads, "3D4", 3.0, 80.0, 0.25, k, k + 47) for k in range(0, 320, 47)]
    assert np.array_equal(full, np.concatenate(parts, axis=1))


def test_tuner_candidates_and_cache(tmp_path):
    """The autotuner's candidate launch shapes (host only) and its cache file: row tiles 32/128/256
    (no 256 with two bases, no tile over twice the rows used), 1/2/4 CTAs per SM, both operand forms
    only for passes of up to 64 simulations; the cache keeps the last valid line per key."""
    from ekgsim_gb300 import _lib as L
    lib = L.load()

    def cands(two, rows, sims):
        out = np.zeros(4 * 64, dtype=np.int32)
        n = ctypes.c_int32()
        L.check(lib.ekg_tune_candidates(two, rows, sims, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 64,
                                        ctypes.byref(n)))
        return [tuple(out[4 * i:4 * i + 4]) for i in range(n.value)]

    big = cands(0, 512, 256)
    assert {c[0] for c in big} == {32, 128, 256} and {c[1] for c in big} == {1, 2, 4}
    assert all(c[2] == 0 for c in big) and {c[3] for c in big} == {0, 4} and len(big) == 18
    assert {c[0] for c in cands(1, 512, 256)} == {32, 128}
    small = cands(0, 2, 1)
    assert {c[0] for c in small} == {32} and {c[2] for c in small} == {0, 1}
    assert all(c[3] == 0 for c in small if c[2] == 1)
    path = str(tmp_path / "tune.txt").encode()
    I4 = ctypes.c_int32 * 4
    L.check(lib.ekg_tune_cache_put(path, b"k1", I4(128, 1, 0, 0), 0.5))
    L.check(lib.ekg_tune_cache_put(path, b"k2", I4(32, 2, 1, 0), 0.25))
    L.check(lib.ekg_tune_cache_put(path, b"k1", I4(256, 4, 0, 4), 0.4))
    with open(path, "a") as f:
        f.write("k1 77 1 0 0.1 9 0\n")  # not a row tile: ignored
    got = I4()
    ms = ctypes.c_double()
    L.check(lib.ekg_tune_cache_get(path, b"k1", got, ctypes.byref(ms)))
    assert tuple(got) == (256, 4, 0, 4) and ms.value == 0.4
    L.check(lib.ekg_tune_cache_get(path, b"k2", got, ctypes.byref(ms)))
    assert tuple(got) == (32, 2, 1, 0)
    assert lib.ekg_tune_cache_get(path, b"k3", got, ctypes.byref(ms)) == -9
    assert lib.ekg_tune_cache_put(path, b"a b", I4(32, 1, 0, 0), 1.0) == -1
