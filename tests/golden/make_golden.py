"""Generate the golden fixtures in tests/golden/ by running the reference itself.

Needs the reference sources ($EKGSIM_REFERENCE, else a checkout named ``reference`` beside this
repository) to build oracle/_ref/ekgSim_ref (the
unmodified ekgSim command line) and oracle/_ref/ref_dump (a driver over the reference's own
simulator library that writes raw FP64 activation times and ECGs); see oracle/build_ref.sh.

Cases (inputs are the seeded synthetic files of ekgsim_gb300.synth, written to a temporary
directory; the reference's test model is used for the last case):
  tiny24      24^3 ellipsoid, 3 layers, 2 leads, 200 steps: raw activation times + raw ECG
              (ref_dump), criteria / violation / result.column (ekgSim_ref -sim ... -out result)
  c64         64^3 ellipsoid, 3 layers, 2 leads, 600 steps: SHA-256 of the activation times,
              raw ECG (ref_dump), criteria / violation / result.column (ekgSim_ref)
  layers10    40^3 ellipsoid, 10 layers with seeded delays, endo-mid-epi interpolation (the
              steepest-descent fit runs for 8 layers), 2 leads, 300 steps: criteria, violation,
              result.column and layer_aps.column (ekgSim_ref -out result -out layer_aps)
  endoepi5    32^3 ellipsoid, 5 layers, endo-epi interpolation, 2 leads, 200 steps: as layers10
  extras24    as tiny24 with the optional criteria on: peak position, the fast approximation as a
              criterion (epi delay 10 ms) and the endo-epi criterion (epi delay 2 ms)
  gate24      as tiny24 with fast approximation limit 0.05, so that the approximation gate skips
              the simulation and the criteria come from the approximation
  rms24, devlin24, vcorr24
              as tiny24 with comparison modes 1 (rms), 3 (devFromLinear) and 4 (vector correlation)
  cube24, n2d4_24
              as tiny24 with the dipole neighbourhoods "cube" (26 neighbours) and "2D4"
  start24     as tiny24 with the simulation starting at 40 ms (the targets are resampled from there)
  k0_24       as tiny24 with resting potentials k0 = -86, -80, -90 in the three base APs (a constant
              term across layers)
  fixed24     as tiny24 with "optimize measuring points = 0" (12 genes, leads at their loaded positions)
  n2d8_24     as tiny24 with the dipole neighbourhood "2D8"
  cells24     as tiny24 with "-out cell_aps 0 3 17 250 100000" (cell APs by the reference's apIndex;
              the last index is out of range and skipped): cell_aps.column values and header lines
  exout24     as tiny24 with "[output files] excitation sequence": the exported sequence text
  exin24      as tiny24 loading a sequence from "[model] excitation sequence" (one the reference
              exported for the same shape with delays {2, 1, 3}) and exporting it again
  model24     the reference's own testRun model (93 x 124 x 124, 24 layers) with the README
              v>=0.1.4 example vector: criteria, violation, result.column (about 3 minutes)

Usage: python tests/golden/make_golden.py [--reference DIR] [--skip-model24] [--only NAME,...]
(--only regenerates the named cases and keeps the others in golden.json)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ekgsim_gb300 import synth  # noqa: E402

README_VECTOR = ("0.00035813,0.0890636,0.0632915,226.183,0.000369406,0.0965625,0.0523254,232.278,"
                 "0.000710767,0.0720323,0.0187579,200.93,23,22,15,13")


def run_cli(ekgsim, wd, genes, outs=("result",)):
    args = [ekgsim, "test", "-sim", ",".join(repr(float(g)) for g in genes)]
    for o in outs:
        args += ["-out", o]
    r = subprocess.run(args, cwd=wd, capture_output=True, text=True)
    m = re.search(r"criteria = <([^>]*)>, violation = (\S+)", r.stdout)
    if not m:
        raise RuntimeError("reference run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    crit = [float(x) for x in m.group(1).split(",")]
    return crit, float(m.group(2))


def read_column_text(path):
    rows = []
    for line in open(path):
        if line.startswith("#") or not line.strip():
            continue
        rows.append([float(x) for x in line.split()])
    return np.array(rows)


def file_head(path):
    return [line.rstrip("\n") for line in open(path) if line.startswith("#")]


def layer_k_hex(path, lk):
    with open(path, "w") as f:
        for row in lk:
            f.write(" ".join(float(v).hex() for v in row) + "\n")


def run_dump(ref_dump, wd, genes, nlayers):
    """Raw activation times and ECG through the reference library (layer APs = base APs with the
    genes substituted, which is what sim.cpp does for three layers)."""
    base = np.array(synth.BASE_AP)
    lk = np.tile(base, (nlayers, 1))
    for i in range(3):
        lk[i if nlayers == 3 else 0, 5:9] = genes[4 * i:4 * i + 4]
    lk_path = os.path.join(wd, "layer_k.txt")
    layer_k_hex(lk_path, lk)
    disp = [repr(float(x)) for x in genes[12:16]]
    r = subprocess.run([ref_dump, "simulator.ini", "dump.bin", "layer_k.txt"] + disp, cwd=wd, capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    raw = open(os.path.join(wd, "dump.bin"), "rb").read()
    nz, ny, nx, nl, st = np.frombuffer(raw[:40], dtype=np.int64)
    at = np.frombuffer(raw[40:40 + 8 * nz * ny * nx], dtype=np.float64).reshape(nz, ny, nx).copy()
    ecg = np.frombuffer(raw[40 + 8 * nz * ny * nx:], dtype=np.float64).reshape(nl, st).copy()
    return at, ecg, lk


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--skip-model24", action="store_true")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    only = set(x for x in args.only.split(",") if x)
    if args.reference is None:
        from oracle.refpath import reference_dir
        args.reference = reference_dir()
    if args.reference is None:
        raise SystemExit("reference sources not found: pass --reference or set EKGSIM_REFERENCE")
    subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "build_ref.sh"), args.reference])
    ekgsim = os.path.join(ROOT, "oracle", "_ref", "ekgSim_ref")
    ref_dump = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    meta = {"generator": "tests/golden/make_golden.py", "cases": {}}
    if only:
        with open(os.path.join(HERE, "golden.json")) as f:
            meta = json.load(f)
    tmp = tempfile.mkdtemp(prefix="ekg_golden_")

    def synth_case(name, spec, steps, nlayers, genes, dump, outs=("result",), raw_at=False, pre_files=None, **ini):
        if only and name not in only:
            return
        wd = os.path.join(tmp, name)
        synth.make_workload(wd, spec, steps, **ini)
        for fname, text in (pre_files or {}).items():
            with open(os.path.join(wd, fname), "w") as f:
                f.write(text)
        crit, viol = run_cli(ekgsim, wd, genes, outs)
        case = {"spec": {"n": spec.n, "semi_axes": list(spec.semi_axes), "wall": spec.wall, "n_layers": nlayers,
                         "delays": list(spec.delays), "n_leads": spec.n_leads, "lead_radius": spec.lead_radius,
                         "n_stim": spec.n_stim, "seed": spec.seed},
                "steps": steps, "ini": {k: v for k, v in ini.items() if k != "base_aps"},
                "genes": [float(g) for g in genes], "criteria": crit, "violation": viol, "outs": list(outs)}
        if pre_files:
            case["files"] = sorted(pre_files)
        if "base_aps" in ini and name not in ("endoepi5",):
            case["base_aps"] = [[float(v) for v in b] for b in ini["base_aps"]]
        arrays = {"result": read_column_text(os.path.join(wd, "result.column"))}
        if "layer_aps" in outs:
            arrays["layer_aps"] = read_column_text(os.path.join(wd, "layer_aps.column"))
        if any(o.startswith("cell_aps") for o in outs):
            arrays["cell_aps"] = read_column_text(os.path.join(wd, "cell_aps.column"))
            arrays["cell_aps_head"] = np.array(file_head(os.path.join(wd, "cell_aps.column")))
        if ini.get("excitation_out"):
            arrays["excitation_out"] = np.array(open(os.path.join(wd, ini["excitation_out"])).read())
        if pre_files:
            for fname, text in pre_files.items():
                arrays["file_" + fname.replace(".", "_")] = np.array(text)
        if dump:
            at, ecg, lk = run_dump(ref_dump, wd, genes, nlayers)
            case["at_sha256"] = hashlib.sha256(at.tobytes()).hexdigest()
            arrays["ecg"] = ecg
            if raw_at:
                arrays["at"] = at
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        meta["cases"][name] = case
        print(name, crit, viol, flush=True)

    s24 = synth.small_spec(24, n_leads=2)
    synth_case("tiny24", s24, 200, 3, synth.genes_for(s24, 0, 0), dump=True, raw_at=True, mid=0.6)
    c0 = synth.config(0)
    synth_case("c64", c0["spec"], 600, 3, synth.genes_for(c0["spec"], 1, 0), dump=True, mid=0.6)
    s10 = synth.HeartSpec(40, (17.5, 15.0, 18.75), 6.0, 10, [1, 2, 3, 1, 2, 3, 1, 2, 3, 2], 2, 44.0, n_stim=3, seed=11)
    synth_case("layers10", s10, 300, 10, synth.genes_for(s10, 3, 9), dump=False, outs=("result", "layer_aps"),
               mid=0.6)
    s5 = synth.HeartSpec(32, (14.0, 12.0, 15.0), 5.0, 5, [1, 2, 2, 1, 3], 2, 36.0, n_stim=3, seed=12)
    g5 = synth.genes_for(s5, 4, 9)
    g5 = np.concatenate([g5[:8], g5[12:16]])  # endo-epi: two gene sets + 2 x 2 lead moves
    synth_case("endoepi5", s5, 200, 5, g5, dump=False, outs=("result", "layer_aps"),
               interpolation="endo-epi", base_aps=(synth.BASE_AP, synth.BASE_AP))
    synth_case("extras24", s24, 200, 3, synth.genes_for(s24, 1, 0), dump=False, mid=0.6, peak=1, fast_is_crit=1,
               endo_epi=2.0)
    synth_case("gate24", s24, 200, 3, synth.genes_for(s24, 2, 0), dump=False, mid=0.6, fast_limit=0.05)
    for i, (name, mode) in enumerate((("rms24", 1), ("devlin24", 3), ("vcorr24", 4))):
        synth_case(name, s24, 200, 3, synth.genes_for(s24, 3 + i, 0), dump=False, mid=0.6, comparison=mode)
    synth_case("cube24", s24, 200, 3, synth.genes_for(s24, 6, 0), dump=False, mid=0.6, nhood="cube")
    synth_case("n2d4_24", s24, 200, 3, synth.genes_for(s24, 7, 0), dump=False, mid=0.6, nhood="2D4")
    synth_case("start24", s24, 200, 3, synth.genes_for(s24, 8, 0), dump=False, mid=0.6, start=40)
    k0_base = tuple([k0] + list(synth.BASE_AP[1:]) for k0 in (-86.0, -80.0, -90.0))
    synth_case("k0_24", s24, 200, 3, synth.genes_for(s24, 9, 0), dump=False, mid=0.6, base_aps=k0_base)
    synth_case("fixed24", s24, 200, 3, synth.genes_for(s24, 10, 0)[:12], dump=False, mid=0.6, optimize_points=0)
    synth_case("n2d8_24", s24, 200, 3, synth.genes_for(s24, 11, 0), dump=False, mid=0.6, nhood="2D8")

    synth_case("cells24", s24, 200, 3, synth.genes_for(s24, 12, 0), dump=False, mid=0.6,
               outs=("result", "cell_aps 0 3 17 250 100000"))
    synth_case("exout24", s24, 200, 3, synth.genes_for(s24, 13, 0), dump=False, mid=0.6,
               excitation_out="es_out.matrix")
    # a sequence computed with other conduction delays ({2, 1, 3} ms), exported by the reference and
    # loaded instead of the heart's own: the run uses the loaded (printed, 3-decimal) times
    if not only or "exin24" in only:
        wd = os.path.join(tmp, "exin24_src")
        other = synth.HeartSpec(s24.n, s24.semi_axes, s24.wall, 3, [2, 1, 3], s24.n_leads, s24.lead_radius,
                                n_stim=s24.n_stim, seed=s24.seed)
        synth.make_workload(wd, other, 200, mid=0.6, excitation_out="es_other.matrix")
        run_cli(ekgsim, wd, synth.genes_for(s24, 14, 0))
        seq = open(os.path.join(wd, "es_other.matrix")).read()
        synth_case("exin24", s24, 200, 3, synth.genes_for(s24, 14, 0), dump=False, mid=0.6,
                   excitation_in="es_in.matrix", excitation_out="es_out.matrix", pre_files={"es_in.matrix": seq})

    if not args.skip_model24 and (not only or "model24" in only):
        wd = os.path.join(tmp, "model24")
        shutil.copytree(os.path.join(args.reference, "testRun"), wd)
        for f in os.listdir(wd):
            os.chmod(os.path.join(wd, f), 0o644)
        genes = [float(x) for x in README_VECTOR.split(",")]
        crit, viol = run_cli(ekgsim, wd, genes)
        np.savez_compressed(os.path.join(HERE, "model24.npz"),
                            result=read_column_text(os.path.join(wd, "result.column")))
        meta["cases"]["model24"] = {"genes": genes, "criteria": crit, "violation": viol,
                                    "source": "reference testRun/ (model_24.matrix, conduction_24.matrix, "
                                              "model_24_measuring_pos.txt, target_ecg_v2_v5.column, simulator.ini)"}
        print("model24", crit, viol, flush=True)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
