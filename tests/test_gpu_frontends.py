"""GPU tests of the drop-in front ends and the served form.

* bin/ekgSim (command-line drop-in) against the reference's own outputs for the same files
  (tests/golden/, made by running the compiled reference): criteria within 1e-4, printed ECG
  rel-L2 <= 1e-4, layer AP curves at print precision, error messages on stdout with exit 0.
* bin/ekgsim_extern (ExternalEvaluation command): input.txt -> output.txt protocol.
* Served form: each result is the same alone and in a mix of concurrent requests on several
  hearts (within the ECG tolerance); admission refusal by free device memory; a malformed request
  fails alone without failing the others in its batch.
"""
import ctypes
import json
import os
import re
import subprocess
import threading

import numpy as np
import pytest

from ekgsim_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "ekgsim_gb300", "bin")
GOLD = os.path.join(ROOT, "tests", "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
TOL = 1e-4


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_case(name, tmp_path):
    c = META["cases"][name]
    s = c["spec"]
    spec = synth.HeartSpec(s["n"], tuple(s["semi_axes"]), s["wall"], s["n_layers"], s["delays"], s["n_leads"],
                           s["lead_radius"], n_stim=s["n_stim"], seed=s["seed"])
    ini = dict(c["ini"])
    if ini.get("interpolation") == "endo-epi":
        ini["base_aps"] = (synth.BASE_AP, synth.BASE_AP)
    if "base_aps" in c:
        ini["base_aps"] = tuple(tuple(b) for b in c["base_aps"])
    synth.make_workload(str(tmp_path), spec, c["steps"], **ini)
    if c.get("files"):
        g = np.load(os.path.join(GOLD, f"{name}.npz"))
        for fname in c["files"]:
            with open(os.path.join(str(tmp_path), fname), "w") as f:
                f.write(str(g["file_" + fname.replace(".", "_")]))
    return c


def read_column(path):
    rows, head = [], []
    for line in open(path):
        if line.startswith("#"):
            head.append(line.rstrip("\n"))
        elif line.strip():
            rows.append([float(x) for x in line.split()])
    return head, np.array(rows)


def run_cli(wd, genes, outs=("result",)):
    args = [os.path.join(BIN, "ekgSim"), "test", "-sim", ",".join(repr(float(g)) for g in genes)]
    for o in outs:
        args += ["-out", o]
    return subprocess.run(args, cwd=wd, capture_output=True, text=True, timeout=300)


@pytest.mark.parametrize("name", ["tiny24", "c64", "layers10", "endoepi5", "extras24", "gate24", "rms24", "devlin24",
                                  "vcorr24", "cube24", "n2d4_24", "start24", "k0_24", "fixed24", "n2d8_24",
                                  "cells24", "exout24", "exin24"])
def test_cli_matches_reference(name, tmp_path):
    c = make_case(name, tmp_path)
    outs = tuple(c.get("outs", ("result", "layer_aps") if name in ("layers10", "endoepi5") else ("result",)))
    r = run_cli(str(tmp_path), c["genes"], outs)
    assert r.returncode == 0
    m = re.search(r" criteria = <([^>]*)>, violation = (\S+)", r.stdout)
    assert m, r.stdout
    crit = np.array([float(x) for x in m.group(1).split(",")])
    assert np.allclose(crit, c["criteria"], rtol=0, atol=TOL)
    assert abs(float(m.group(2)) - c["violation"]) <= 1e-6 * max(1.0, abs(c["violation"]))
    assert r.stdout.rstrip().endswith("All done")
    assert "simulation done in" in r.stdout
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    head, res = read_column(os.path.join(str(tmp_path), "result.column"))
    assert head[0].startswith("#Comment: input=<") and head[-1].startswith("#Time[ms]\t")
    if g["result"].size == 0:  # the fast-approximation gate skipped the simulation: headers only
        assert res.size == 0
        return
    assert res.shape == g["result"].shape
    assert np.allclose(res[:, 0], g["result"][:, 0])
    assert rel_l2(res[:, 1:], g["result"][:, 1:]) <= TOL
    assert os.path.exists(os.path.join(str(tmp_path), "target_chk.column"))
    if "layer_aps" in outs:
        _, aps = read_column(os.path.join(str(tmp_path), "layer_aps.column"))
        ref = g["layer_aps"]
        assert aps.shape == ref.shape
        assert np.all(np.abs(aps[:, 1:] - ref[:, 1:]) <= 2e-5 * np.abs(ref[:, 1:]) + 1e-9)
    if "cell_aps" in g:
        # cell APs by the reference's apIndex: header lines (k vectors printed with 6 digits) and values
        head, aps = read_column(os.path.join(str(tmp_path), "cell_aps.column"))
        assert head == [str(x) for x in g["cell_aps_head"]]
        ref = g["cell_aps"]
        assert aps.shape == ref.shape
        assert np.all(np.abs(aps[:, 1:] - ref[:, 1:]) <= 2e-5 * np.abs(ref[:, 1:]) + 1e-9)
    if "excitation_out" in g:
        # [output files] excitation sequence: the same text as the reference's export
        ini = c["ini"]
        with open(os.path.join(str(tmp_path), ini["excitation_out"])) as f:
            assert f.read() == str(g["excitation_out"])


def test_cli_errors_print_and_exit_zero(tmp_path):
    c = make_case("tiny24", tmp_path)
    r = run_cli(str(tmp_path), c["genes"][:7])  # too few genes (sim.cpp:458-459)
    assert r.returncode == 0
    assert "runtime error caught: Solution does not contain enough values" in r.stdout
    r = run_cli(str(tmp_path), list(c["genes"]) + [1.0])  # too many (sim.cpp:835-841)
    assert r.returncode == 0
    assert "runtime error caught: chromosome size does not agree" in r.stdout
    os.remove(os.path.join(str(tmp_path), "leads.txt"))
    r = run_cli(str(tmp_path), c["genes"])
    assert r.returncode == 0 and "failed to open file containing measuring points" in r.stdout


def test_extern_adapter(tmp_path):
    c = make_case("tiny24", tmp_path)
    d = tmp_path / "process0"
    d.mkdir()
    with open(d / "input.txt", "w") as f:
        f.write("# file generated by ExternalEvaluation class\n")
        for v in c["genes"]:
            f.write(f"{v}\n")
    r = subprocess.run([os.path.join(BIN, "ekgsim_extern"), str(d)], cwd=str(tmp_path), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    vals, viol = [], None
    for line in open(d / "output.txt"):
        if line.startswith("#"):
            parts = line[1:].split()
            if parts and parts[0] == "violation":
                viol = float(parts[1])
        elif line.strip():
            vals.append(float(line))
    assert np.allclose(vals, c["criteria"], rtol=0, atol=TOL)
    assert viol == pytest.approx(c["violation"], abs=1e-9)
    with open(d / "input.txt", "w") as f:
        f.write("# too few genes\n0.0005\n")
    r = subprocess.run([os.path.join(BIN, "ekgsim_extern"), str(d)], cwd=str(tmp_path), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode != 0


def _served_heart(engine, n, seed):
    from ekgsim_gb300.engine import Heart
    spec = synth.small_spec(n, n_leads=4, seed=seed)
    grid = synth.ellipsoid_heart(spec)
    tm = synth.transfer_matrix(3, spec.delays)
    leads = synth.leads(spec, np.random.Generator(np.random.PCG64(seed)))[:, ::-1].copy()
    h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, 300.0, 1.0)
    h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
               [t for t in synth.analytic_target(4, 300, seed)], mid_position=0.6)
    return h, spec


def test_served_same_alone_and_in_mix(engine):
    from ekgsim_gb300.engine import Server
    hearts = [_served_heart(engine, n, 40 + n) for n in (20, 28, 36)]
    srv = Server(engine, max_batch=64, max_wait_us=2000)
    ids = [srv.add_heart(h) for h, _ in hearts]
    probe = synth.genes_for(hearts[1][1], 7, 3)
    rid = srv.submit(ids[1], probe)
    alone = srv.poll(rid, ids[1], wait_ms=60000, want_ecg=True)
    assert alone is not None
    # the same request inside a mix of concurrent submissions on all hearts
    reqs = []
    lock = threading.Lock()

    def client(k):
        for j in range(12):
            hid = (k + j) % 3
            g = synth.genes_for(hearts[hid][1], 100 + 13 * k + j, 3)
            r = srv.submit(ids[hid], g)
            with lock:
                reqs.append((r, hid))

    ths = [threading.Thread(target=client, args=(k,)) for k in range(4)]
    for t in ths:
        t.start()
    rid2 = srv.submit(ids[1], probe)
    for t in ths:
        t.join()
    mixed = srv.poll(rid2, ids[1], wait_ms=60000, want_ecg=True)
    batches = []
    for r, hid in reqs:
        out = srv.poll(r, hid, wait_ms=60000)
        assert out is not None
        batches.append(out[3]["batch"])
    assert max(batches + [mixed[3]["batch"]]) > 1  # requests were packed together
    assert rel_l2(mixed[2], alone[2]) <= TOL
    assert np.allclose(mixed[0], alone[0], rtol=0, atol=TOL)
    assert mixed[1] == alone[1]
    srv.close()


def test_served_admission_refused_and_bad_request_isolated(engine):
    from ekgsim_gb300 import _lib as L
    from ekgsim_gb300.engine import EkgError, Server
    h, spec = _served_heart(engine, 20, 5)
    srv = Server(engine, max_batch=16, max_wait_us=5000)
    hid = srv.add_heart(h)
    # a malformed request in the same batch as good ones fails alone
    good = [srv.submit(hid, synth.genes_for(spec, r, 5)) for r in range(3)]
    bad = srv.submit(hid, np.zeros(3))
    for r in good:
        assert srv.poll(r, hid, wait_ms=60000) is not None
    with pytest.raises(EkgError) as e:
        srv.poll(bad, hid, wait_ms=60000)
    assert e.value.code == -1
    # no free device memory: admission refused with EKG_ERR_OUT_OF_MEMORY
    FREE = ctypes.CFUNCTYPE(ctypes.c_uint64, ctypes.c_void_p)
    zero = FREE(lambda ctx: 0)
    L.check(L.load().ekg_server_set_free_bytes_provider(srv._h, ctypes.cast(zero, ctypes.c_void_p), None))
    srv2_h = srv  # same server, new requests
    r = srv2_h.submit(hid, synth.genes_for(spec, 9, 5))
    with pytest.raises(EkgError) as e:
        srv2_h.poll(r, hid, wait_ms=60000)
    assert e.value.code == -2
    L.check(L.load().ekg_server_set_free_bytes_provider(srv._h, None, None))
    r = srv.submit(hid, synth.genes_for(spec, 10, 5))
    assert srv.poll(r, hid, wait_ms=60000) is not None
    srv.close()


def test_served_c4_hearts_match_oracle(engine):
    """The served configuration's four hearts (48^3, 96^3, 144^3, 192^3 scaled ellipsoids, 3 layers,
    12 leads, 600 steps) through the served path: activation times bitwise per heart; per heart a
    probe request alone and again inside a concurrent mix on all hearts, and one more request of the
    mix, each against the FP64 oracle."""
    from ekgsim_gb300.engine import Heart, Server
    from oracle import oracle as O
    cfg = synth.config(3)
    steps = cfg["steps"]
    hearts = []
    for spec in cfg["hearts"]:
        grid = synth.ellipsoid_heart(spec)
        tm = synth.transfer_matrix(spec.n_layers, spec.delays)
        leads = synth.leads(spec, np.random.Generator(np.random.PCG64(spec.seed)))[:, ::-1].copy()
        h = Heart.create(engine, grid, tm, leads, "3D4", 0.0, float(steps), 1.0)
        target = [t for t in synth.analytic_target(spec.n_leads, steps, spec.seed + 999)]
        h.set_eval([synth.BASE_AP] * 3, synth.K_MIN, synth.K_MAX, [5, 6, 7, 8], target, mid_position=0.6)
        hearts.append((h, spec, grid, tm, leads, target))
    srv = Server(engine, max_batch=64, max_wait_us=1000)
    ids = [srv.add_heart(x[0]) for x in hearts]
    probes = [synth.genes_for(x[1], 900 + k, 3) for k, x in enumerate(hearts)]
    alone = [srv.poll(srv.submit(ids[k], probes[k]), ids[k], wait_ms=120000, want_ecg=True) for k in range(4)]
    reqs = []
    lock = threading.Lock()

    def client(c):
        for j in range(8):
            k = (c + j) % 4
            g = synth.genes_for(hearts[k][1], 1000 + 37 * c + j, 3)
            r = srv.submit(ids[k], g)
            with lock:
                reqs.append((r, k, g))

    ths = [threading.Thread(target=client, args=(c,)) for c in range(4)]
    for t in ths:
        t.start()
    mixed_ids = [srv.submit(ids[k], probes[k]) for k in range(4)]
    for t in ths:
        t.join()
    mixed = [srv.poll(mixed_ids[k], ids[k], wait_ms=120000, want_ecg=True) for k in range(4)]
    others = {}
    for r, k, g in reqs:
        out = srv.poll(r, ids[k], wait_ms=120000, want_ecg=True)
        assert out is not None
        others.setdefault(k, (g, out))
    srv.close()
    for k, (h, spec, grid, tm, leads, target) in enumerate(hearts):
        at, layer = O.activation(grid, tm)
        assert np.array_equal(h.activation().view(np.int64), at.view(np.int64)), spec.n
        for g, out in ((probes[k], alone[k]), (probes[k], mixed[k]), others[k]):
            lk = O.layer_aps(3, np.array([synth.BASE_AP] * 3), synth.K_MIN, synth.K_MAX, [5, 6, 7, 8],
                             "endo-mid-epi", 0.6, g[:12])[0]
            moved = O.move_leads(leads, g[12:].reshape(-1, 2))
            ref = O.run(layer, at, lk, moved, "3D4", 0.0, float(steps), 1.0)
            assert rel_l2(out[2], ref) <= TOL, spec.n
            for l in range(spec.n_leads):
                assert out[0][l] == pytest.approx(O.clamp(O.compare(2, ref[l], target[l])), abs=1e-4)
        h.close()


def test_served_many_and_criteria_only(engine):
    """submit_many / poll_many hand over the same criteria as single submissions and polls; a server
    without ECGs answers an ECG poll with an error; bad requests in a burst fail alone."""
    from ekgsim_gb300.engine import EkgError, Server
    hs = [_served_heart(engine, n, 60 + n) for n in (20, 28)]
    srv = Server(engine, max_batch=32, max_wait_us=500, keep_ecg=False)
    ids = [srv.add_heart(h) for h, _ in hs]
    _, nc = hs[0][0].eval_shape()
    genes = np.stack([synth.genes_for(hs[i % 2][1], 200 + i, 3) for i in range(24)])
    hid = np.array([ids[i % 2] for i in range(24)], dtype=np.int32)
    bad = genes.copy()
    bad[5, 3] = np.nan
    rids = srv.submit_many(hid, bad)
    status, crit, viol, total, batch = srv.poll_many(rids, nc, wait_ms=120000)
    assert status[5] == -1 and (np.delete(status, 5) == 0).all()
    assert batch.max() > 1
    for i in (0, 7, 23):
        h = hs[i % 2][0]
        c1, v1 = h.eval(genes[i])[:2]
        assert np.allclose(crit[i], c1, rtol=0, atol=TOL)
        assert viol[i] == v1
    r = srv.submit(ids[0], genes[0])
    with pytest.raises(EkgError):
        srv.poll(r, ids[0], wait_ms=120000, want_ecg=True)
    srv.close()
