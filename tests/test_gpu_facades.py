"""GPU tests of the C++ and Python facades, run as the reference's callers would use them, against
the reference's own outputs (tests/golden/):

* tests/facade/facade_check.cpp (compiled here) drives ekgsim::Evaluation (operator(),
  simulationDone, evaluateBatch), GpuOptimizationFunction through a VirtualOptimizationFunction
  reference, GenerationQueue over a master with AMS-DEMO's job interface, and ekgsim::EkgSim
  (loadFromIni, setAps, setMeasuringPoints, run, getMeasurement);
* ekgsim_gb300.simulator (OptimizationFunction, EkgSim) the same way from Python.
Bars: criteria within 1e-4 of the reference's, violations equal, ECG rel-L2 <= 1e-4."""
import json
import os
import subprocess

import numpy as np
import pytest

from ekgsim_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
LIBDIR = os.path.join(ROOT, "ekgsim_gb300")
TOL = 1e-4


def make_case(name, wd):
    c = META["cases"][name]
    s = c["spec"]
    spec = synth.HeartSpec(s["n"], tuple(s["semi_axes"]), s["wall"], s["n_layers"], s["delays"], s["n_leads"],
                           s["lead_radius"], n_stim=s["n_stim"], seed=s["seed"])
    synth.make_workload(str(wd), spec, c["steps"], **dict(c["ini"]))
    return c, spec


@pytest.fixture(scope="module")
def facade_bin(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("facade") / "facade_check")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "facade", "facade_check.cpp"), "-o", out, "-L", LIBDIR,
                        "-lekgsim_gb300", f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run_facade(binary, wd, genes):
    with open(os.path.join(str(wd), "genes.txt"), "w") as f:
        for g in genes:
            f.write(",".join(repr(float(x)) for x in g) + "\n")
    r = subprocess.run([binary], cwd=str(wd), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        p = line.split()
        out.setdefault(p[0], {})[int(p[1])] = [float(x) for x in p[2:]]
    return out


@pytest.mark.parametrize("name", ["tiny24", "gate24", "fixed24"])
def test_cpp_facades_match_reference(facade_bin, name, tmp_path):
    c, spec = make_case(name, tmp_path)
    g0 = np.array(c["genes"])
    extra = [synth.genes_for(spec, 40 + k, 0)[:g0.size] for k in range(4)]
    genes = [g0] + extra
    out = run_facade(facade_bin, tmp_path, genes)
    nc = len(c["criteria"])
    single = out["single"]
    assert np.allclose(single[0][:nc], c["criteria"], rtol=0, atol=TOL)
    assert single[0][nc] == pytest.approx(c["violation"], abs=1e-9)
    # simulationDone: the approximation gate of gate24 skips the simulation (sim.cpp:712-748)
    assert int(single[0][nc + 1]) == (0 if name == "gate24" else 1)
    for tag in ("batch", "plugin", "queue"):
        assert sorted(out[tag]) == list(range(len(genes))), tag
        for i in range(len(genes)):
            assert np.allclose(out[tag][i][:nc], single[i][:nc], rtol=0, atol=TOL), (tag, i)
            assert out[tag][i][nc] == single[i][nc], (tag, i)
    for i in range(len(genes)):
        d, m = out["ecg"][i]
        assert d <= TOL * m, i


def test_python_facades_match_reference(tmp_path):
    from ekgsim_gb300 import simulator as S
    from oracle import oracle as O
    c, spec = make_case("tiny24", tmp_path)
    ini = os.path.join(str(tmp_path), "simulator.ini")
    f = S.OptimizationFunction(ini, out_dir=str(tmp_path))
    crit, viol = f(c["genes"])
    assert np.allclose(crit, c["criteria"], rtol=0, atol=TOL)
    assert viol == pytest.approx(c["violation"], abs=1e-9)
    assert f.simulation_done()
    ng, nc, lo, hi = f.get_gene_params()
    assert ng == len(c["genes"]) and nc == len(c["criteria"])
    genes = np.stack([np.array(c["genes"])] + [synth.genes_for(spec, 50 + k, 0) for k in range(3)])
    cb, vb = f.evaluate_batch(genes)
    assert np.allclose(cb[0], c["criteria"], rtol=0, atol=TOL)
    assert f.normalize([-1e9] * ng) == list(lo)
    # SimLib::EkgSim sequence (simlib/sim_lib.h:78-92): settings, model, APs, run, measurements
    s = O.load_setup(str(tmp_path))
    _, _, ecg_ref, lk, leads = O.evaluate(s, np.array(c["genes"]))
    sim = S.EkgSim()
    sim.loadSettings(ini)
    sim.simExcitationSequence()
    assert sim.requiredAps() == lk.shape[0]
    sim.setApsDestructive(lk)
    sim.moveMeasuringPoints(np.array(c["genes"][12:16]).reshape(2, 2), s.leads_zyx)
    sim.run()
    ecg = np.stack([sim.getMeasurement(i) for i in range(sim.numMeasurements())])
    assert float(np.linalg.norm(ecg - ecg_ref) / np.linalg.norm(ecg_ref)) <= TOL
    assert np.array_equal(sim.activationTimes().ravel().view(np.int64), s.at.ravel().view(np.int64))
