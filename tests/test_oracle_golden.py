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


def _write_pre_files(name, tmp_path):
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    for fname in META["cases"][name].get("files", []):
        with open(os.path.join(str(tmp_path), fname), "w") as f:
            f.write(str(g["file_" + fname.replace(".", "_")]))
    return g


@pytest.mark.skipif("cells24" not in META["cases"], reason="no golden")
def test_cell_aps_output(tmp_path):
    """-out "cell_aps 0 3 17 250 100000": the cell APs with those reference apIndex numbers (first
    appearance in raster order, simlib/simulator.cpp:570-590; the out-of-range one skipped), their
    k vectors (k8 shifted by the activation time) in the header and their values at t = 0..699."""
    c, s = make_case("cells24", tmp_path)
    g = np.load(os.path.join(GOLD, "cells24.npz"))
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    idx, al, aa = O.ap_indices(s.layer, s.at)
    rows = g["cell_aps"]
    assert rows.shape == (700, 5)
    for j, a in enumerate((0, 3, 17, 250)):
        k = lk[al[a] - 1].copy()
        got = np.array([O.wohl(np.concatenate([k[:8], [k[8] - aa[a]]]), float(t) - aa[a]) for t in range(700)])
        assert printed_close(got, rows[:, 1 + j], atol=1e-9), a


@pytest.mark.skipif("exout24" not in META["cases"], reason="no golden")
def test_excitation_sequence_export(tmp_path):
    """[output files] excitation sequence: the exported text (simlib/simulator.cpp:71-106) equals
    the reference's byte for byte."""
    c, s = make_case("exout24", tmp_path)
    g = np.load(os.path.join(GOLD, "exout24.npz"))
    assert O.export_excitation(s.at) == str(g["excitation_out"])


@pytest.mark.skipif("exin24" not in META["cases"], reason="no golden")
def test_excitation_sequence_load(tmp_path):
    """[model] excitation sequence: the run uses the loaded 3-decimal times (here a sequence of
    other conduction delays) instead of the automaton's; criteria, printed ECG and the re-export
    match the reference."""
    c = META["cases"]["exin24"]
    g = _write_pre_files("exin24", tmp_path)
    c, s = make_case("exin24", tmp_path)
    crit, viol, ecg, lk, leads = O.evaluate(s, np.array(c["genes"]))
    assert printed_close(crit, np.array(c["criteria"]))
    assert printed_close(ecg.T, g["result"][:, 1:])
    assert O.export_excitation(s.at) == str(g["excitation_out"])
    at_ca, _ = O.activation(s.raw, s.tm)
    assert not np.array_equal(at_ca, s.at)  # the loaded sequence is not the heart's own
