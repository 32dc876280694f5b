"""The FP64 oracle pinned against outputs of the reference itself (tests/golden/, made by
tests/golden/make_golden.py from the compiled reference).

Raw FP64 activation times and ECGs (from a driver over the reference's simulator library) must
match bit for bit; values the reference prints with 6 significant digits (criteria, result.column,
layer_aps.column) must match to that precision.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from ekgsim_gb300 import synth
from oracle import oracle as O
from oracle.refpath import reference_dir

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
META = json.load(open(os.path.join(GOLD, "golden.json")))
SYNTH_CASES = [c for c in ("tiny24", "c64", "layers10", "endoepi5", "rms24", "devlin24", "vcorr24", "cube24",
                           "n2d4_24", "start24", "k0_24", "fixed24", "n2d8_24") if c in META["cases"]]
PRINT_RTOL = 1e-5  # %e with 6 significant digits


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
    return c, O.load_setup(str(tmp_path))


def printed_close(got, ref, rtol=PRINT_RTOL, atol=1e-12):
    return np.all(np.abs(got - ref) <= rtol * np.abs(ref) + atol)


@pytest.mark.parametrize("name", [c for c in ("tiny24", "c64") if c in META["cases"]])
def test_bit_exact_activation_and_ecg(name, tmp_path):
    c, s = make_case(name, tmp_path)
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    assert hashlib.sha256(s.at.tobytes()).hexdigest() == c["at_sha256"]
    if "at" in g:
        assert np.array_equal(s.at.view(np.int64), g["at"].view(np.int64))
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    assert np.array_equal(ecg.view(np.int64), g["ecg"].view(np.int64))


@pytest.mark.parametrize("name", SYNTH_CASES)
def test_criteria_and_printed_ecg(name, tmp_path):
    c, s = make_case(name, tmp_path)
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    assert printed_close(crit, np.array(c["criteria"]))
    assert printed_close(np.array([viol]), np.array([c["violation"]]))
    res = g["result"]
    assert res.shape == (ecg.shape[1], 1 + ecg.shape[0])
    assert np.allclose(res[:, 0], s.start + np.arange(ecg.shape[1]) * s.dt)
    assert printed_close(ecg.T, res[:, 1:])


@pytest.mark.parametrize("name", [c for c in ("extras24", "gate24") if c in META["cases"]])
def test_optional_criteria_and_approximation_gate(name, tmp_path):
    """extras24: peak position, fast approximation and endo-epi criteria together (the reference
    writes the approximation at index n_leads, where the peak pairs then overwrite it); gate24: the
    approximation gate skips the simulation, the criteria come from the approximation and the
    reference writes no ECG rows."""
    c, s = make_case(name, tmp_path)
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    assert crit.shape == (len(c["criteria"]),)
    assert printed_close(crit, np.array(c["criteria"]))
    if name == "gate24":
        assert g["result"].size == 0
    else:
        assert printed_close(ecg.T, g["result"][:, 1:])


@pytest.mark.parametrize("name", [c for c in ("layers10", "endoepi5") if c in META["cases"]])
def test_layer_aps_from_genes(name, tmp_path):
    """Gene -> layer AP construction incl. the steepest-descent interpolation (sim.cpp:751-916),
    checked through the layer AP curves the reference writes (-out layer_aps, t = 0..699)."""
    c, s = make_case(name, tmp_path)
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    curves = g["layer_aps"]
    assert curves.shape[1] == 1 + lk.shape[0]
    for i in range(lk.shape[0]):
        got = np.array([O.wohl(lk[i], float(t)) for t in range(700)])
        assert printed_close(got, curves[:, 1 + i], atol=1e-9), i


@pytest.mark.skipif(reference_dir() is None or "model24" not in META["cases"],
                    reason="the reference's test model is not present")
def test_reference_test_model_24_layers(tmp_path):
    """The reference's own test model (93 x 124 x 124, 24 layers, 555,868 voxels) with the README
    example vector: criteria, violation and the full printed ECG."""
    import shutil
    wd = str(tmp_path / "testRun")
    shutil.copytree(os.path.join(reference_dir(), "testRun"), wd)
    for f in os.listdir(wd):
        os.chmod(os.path.join(wd, f), 0o644)
    c = META["cases"]["model24"]
    s = O.load_setup(wd)
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    assert printed_close(crit, np.array(c["criteria"]))
    assert printed_close(np.array([viol]), np.array([c["violation"]]))
    res = np.load(os.path.join(GOLD, "model24.npz"))["result"]
    assert printed_close(ecg.T, res[:, 1:])
