"""Seeded synthetic EkgSim workloads, written in the reference's own file formats.

No public data set is involved: every heart, lead set, parameter vector and target is
generated from a numpy ``PCG64(seed)`` stream, with seed = config index * 1000 + request
index.  The files match what the reference simulator reads:

* ``.matrix`` heart model: ``3d X x Y x Z space`` header, data z-slowest / x-fastest,
  layer ids 1..nL, 0 = empty, negative = stimulus voxel
  (simlib/matrix.h:125-129 shapeLoad, :134-248 importMatrix);
* conduction (transfer) matrix: ``2d n x n tab``, (nL+1)^2 entries in ms, row/column 0
  unused (testRun/conduction_24.matrix:1-4);
* measuring points: one ``x, y, z`` line per lead (simlib/simulator.cpp:369-388);
* ``simulator.ini`` with the reference's section and key names (simlib/simulator.h:107-145,
  SimSettings.h:158-356);
* target ``.column``: time column + one column per lead (simlib/columnFile.h:86-186).

Heart geometry: a thick-walled ellipsoid ventricle.  Voxel (z, y, x) of an N^3 grid has centre
c = i + 0.5 - N/2 per axis; it belongs to the wall when it lies inside the outer ellipsoid
(ax, ay, az) and outside the inner one (ax - w, ay - w, az - w).  The wall is split into nL
layers by nested ellipsoids at semi-axes a - k*w/nL: layer 1 (endocardium) is innermost,
layer nL (epicardium) outermost.  The stimulus is the ``n_stim`` layer-1 voxels with the
smallest z (apex at the -z pole), ties broken by x^2 + y^2 and then by linear index.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

# README.md:102-103 (v>=0.1.4): 3 x (k5, k6, k7, k8) then 2 x 2 lead displacements
GENE_MIN = np.array([0.0003, 0.01, 0.01, 200.0] * 3 + [-50.0] * 4)
GENE_MAX = np.array([0.0010, 0.10, 0.10, 400.0] * 3 + [50.0] * 4)

# testRun/simulator.ini:48-50 base APs (all three equal there)
BASE_AP = [0.0, 2.5, 100.0, 0.90, 0.1, 0.0010, 0.10, 0.10, 250.0]
# k bounds chosen equal to the README gene bounds so that violation = 0
K_MIN = [0.0, 1.5, 100.0, 0.85, 0.05, 0.0003, 0.01, 0.01, 200.0]
K_MAX = [0.0, 3.5, 100.0, 0.95, 0.2, 0.0010, 0.10, 0.10, 400.0]


@dataclass
class HeartSpec:
    """One synthetic heart: grid size, ellipsoid, layers, conduction delays, leads."""
    n: int
    semi_axes: Tuple[float, float, float]  # (ax, ay, az) outer semi-axes in voxels
    wall: float
    n_layers: int
    delays: Sequence[float]  # per destination layer, ms (transfer matrix T[s][d] = delays[d-1])
    n_leads: int
    lead_radius: float
    lead_surface: str = "sphere"  # "sphere" or "torso" (ellipsoid of 1.2x the heart)
    n_stim: int = 5
    seed: int = 0

    @property
    def shape(self):
        return (self.n, self.n, self.n)


def ellipsoid_heart(spec: HeartSpec) -> np.ndarray:
    """Signed layer grid [z][y][x] (int16): 0 empty, 1..nL layers, negative = stimulus."""
    n = spec.n
    ax, ay, az = spec.semi_axes
    w = spec.wall
    c = np.arange(n, dtype=np.float64) + 0.5 - n / 2.0
    z = c[:, None, None]
    y = c[None, :, None]
    x = c[None, None, :]

    def inside(sx, sy, sz):
        return (x / sx) ** 2 + (y / sy) ** 2 + (z / sz) ** 2 <= 1.0

    grid = np.zeros((n, n, n), dtype=np.int16)
    outer = inside(ax, ay, az)
    inner = inside(ax - w, ay - w, az - w)
    wall = outer & ~inner
    # depth band j (0 = outermost) -> layer nL - j
    band = np.zeros((n, n, n), dtype=np.int16)
    for k in range(1, spec.n_layers):
        d = k * w / spec.n_layers
        band += inside(ax - d, ay - d, az - d).astype(np.int16)
    grid[wall] = (spec.n_layers - band[wall]).astype(np.int16)
    # stimulus: n_stim layer-1 voxels with minimal z, ties by x^2+y^2 then linear index
    zi, yi, xi = np.nonzero(grid == 1)
    lin = (zi * n + yi) * n + xi
    r2 = c[xi] ** 2 + c[yi] ** 2
    order = np.lexsort((lin, r2, zi))
    pick = order[: spec.n_stim]
    grid[zi[pick], yi[pick], xi[pick]] *= -1
    return grid


def transfer_matrix(n_layers: int, delays: Sequence[float]) -> np.ndarray:
    """Conduction matrix: row/col 0 = -1, T[s][d] = delays[d-1] for s, d >= 1.  It is padded
    with -1 to at least 12 x 12, because the reference checks the matrix size against its
    default of 12 layers before the model is loaded (sim.cpp:372 runs loadTransferMatrix
    before loadShape; simlib/simulator.cpp:201-206, simlib/simulator.h:532)."""
    size = max(n_layers + 1, 12)
    t = np.full((size, size), -1.0)
    for s in range(1, n_layers + 1):
        for d in range(1, n_layers + 1):
            t[s, d] = float(delays[d - 1])
    return t


def leads(spec: HeartSpec, rng: np.random.Generator) -> np.ndarray:
    """Lead positions as (L, 3) x, y, z in file coordinates (voxel units from the (0,0,0) corner)."""
    v = rng.normal(size=(spec.n_leads, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    centre = np.full(3, spec.n / 2.0)
    if spec.lead_surface == "torso":
        ax, ay, az = spec.semi_axes
        scale = 1.2 * np.array([ax, ay, az])
        # point on the ellipsoid along direction v
        t = 1.0 / np.sqrt(((v / scale) ** 2).sum(axis=1))
        return centre + v * t[:, None]
    return centre + spec.lead_radius * v


def draw_genes(rng: np.random.Generator, n_leads: int) -> np.ndarray:
    """16 README-bounded genes, then zeros so the vector has the 12 + 2L genes the reference
    expects when all L leads are movable (sim.cpp:835-841); leads 2..L-1 stay in place."""
    g = GENE_MIN + (GENE_MAX - GENE_MIN) * rng.random(16)
    if n_leads > 2:
        g = np.concatenate([g, np.zeros(2 * (n_leads - 2))])
    return g


def layer_delays(n_layers: int, rng: np.random.Generator) -> List[float]:
    return [float(v) for v in rng.integers(1, 4, size=n_layers)]


# ---------------------------------------------------------------- configurations
def config(index: int) -> dict:
    """The five workload configurations (index 0..4) by their sizes."""
    if index == 0:
        spec = HeartSpec(64, (28, 24, 30), 6, 3, [1, 2, 2], 2, 60.0, seed=0)
        return dict(name="plain-fp64-64cube", spec=spec, steps=600, batch=1)
    if index == 1:
        spec = HeartSpec(128, (56, 48, 60), 12, 3, [1, 2, 2], 12, 120.0, seed=1000)
        return dict(name="single-128cube-12lead", spec=spec, steps=600, batch=1)
    if index == 2:
        spec = HeartSpec(160, (70, 60, 75), 14, 3, [1, 2, 2], 12, 120.0, seed=2000)
        return dict(name="batched-160cube-256sims", spec=spec, steps=600, batch=256)
    if index == 3:
        hearts = []
        for j, f in enumerate((0.75, 1.5, 2.25, 3.0)):
            n = int(round(64 * f))
            hearts.append(HeartSpec(n, (28 * f, 24 * f, 30 * f), 6 * f, 3, [1, 2, 2], 12, 120.0,
                                    seed=3000 + 100 * j))
        return dict(name="served-4hearts", hearts=hearts, steps=600, rate=500.0)
    if index == 4:
        rng = np.random.Generator(np.random.PCG64(4000))
        spec = HeartSpec(256, (112, 96, 120), 24, 10, layer_delays(10, rng), 64, 0.0,
                         lead_surface="torso", seed=4000)
        return dict(name="bsm-256cube-64lead", spec=spec, steps=800, batch=64)
    raise ValueError(index)


def small_spec(n: int = 16, n_layers: int = 3, n_leads: int = 2, seed: int = 7) -> HeartSpec:
    """Tiny ellipsoid for exhaustive checks (semi-axes scale with n)."""
    f = n / 64.0
    return HeartSpec(n, (28 * f, 24 * f, 30 * f), max(2.0, 6 * f), n_layers,
                     [1, 2, 2] if n_layers == 3 else [1 + (i % 3) for i in range(n_layers)],
                     n_leads, 60.0 * f + 4, n_stim=min(5, 3), seed=seed)


# ---------------------------------------------------------------- file writers
def write_matrix(path: str, grid: np.ndarray, comment: str = "synthetic ellipsoid ventricle") -> None:
    """Shape file in the reference's text format (space separated, z blocks)."""
    nz, ny, nx = grid.shape
    with open(path, "w") as f:
        f.write(f"# {comment}\n")
        f.write(f"3d {nx} x {ny} x {nz} space\n")
        for zz in range(nz):
            rows = [" ".join(str(int(v)) for v in grid[zz, yy]) for yy in range(ny)]
            f.write("\n".join(rows))
            f.write("\n\n")


def write_transfer(path: str, t: np.ndarray) -> None:
    n = t.shape[0]
    with open(path, "w") as f:
        f.write("Conduction matrix\n")
        f.write(f"2d {n} x {n} tab\n")
        for row in t:
            f.write("\t".join(repr(float(v)) if v != int(v) else str(int(v)) for v in row))
            f.write("\n")


def write_points(path: str, pts_xyz: np.ndarray) -> None:
    with open(path, "w") as f:
        for p in pts_xyz:
            f.write(f"{float(p[0])!r}, {float(p[1])!r}, {float(p[2])!r}\n")


def write_column(path: str, start: float, dt: float, columns: np.ndarray, names=None) -> None:
    """``#``-commented header, then rows of time + one value per column (full precision)."""
    columns = np.atleast_2d(columns)
    with open(path, "w") as f:
        f.write("# synthetic target ECG\n")
        f.write("#Time[ms]\t" + "\t".join(names or [f"lead{i}" for i in range(columns.shape[0])]) + "\n")
        for i in range(columns.shape[1]):
            f.write(repr(start + i * dt) + "\t" + "\t".join(repr(float(v)) for v in columns[:, i]) + "\n")


def ini_text(shape="model.matrix", transfer="conduction.matrix", points="leads.txt",
             targets="target.column", start=0, length=600, dt=1, nhood="3D4",
             base_aps=(BASE_AP, BASE_AP, BASE_AP), k_min=K_MIN, k_max=K_MAX,
             free_k=(5, 6, 7, 8), optimize_points=1, comparison=2, mid=0.6,
             interpolation="endo-mid-epi", fast_limit=2, fast_is_crit=0, fast_delay=10.0, peak=0,
             endo_epi=-0.5, extra_opt: str = "", excitation_in: str = "", excitation_out: str = "") -> str:
    """simulator.ini text.  excitation_in / excitation_out set the "excitation sequence" keys of
    [model] (load a precomputed sequence instead of computing it) and [output files] (write the
    sequence, simlib/simulator.h:107-145)."""
    def vec(v):
        return ", ".join(repr(float(x)) for x in v)
    lines = [
        "[model]",
        f"shape = {shape}",
        f"transfer = {transfer}",
        f"points = {points}",
    ]
    if excitation_in:
        lines.append(f"excitation sequence = {excitation_in}")
    lines += [
        "",
        "[output files]",
        "results filename = result.column",
    ]
    if excitation_out:
        lines.append(f"excitation sequence = {excitation_out}")
    lines += [
        "",
        "[simulation]",
        f"start = {start}",
        f"length = {length}",
        f"neighbourhood type = {nhood}",
        f"time step = {dt}",
        "",
        "[measuring points]",
        "displacement min = -50",
        "displacement max = 50",
        "",
        "[wohlfart ap]",
        f"interpolation = {interpolation}",
        f"mid AP position = {mid}",
    ]
    for i, b in enumerate(base_aps):
        lines.append(f"base ap {i + 1} = {vec(b)}")
    lines += [
        f"k min = {vec(k_min)}",
        f"k max = {vec(k_max)}",
        "free k = " + ", ".join(str(k) for k in free_k),
        "",
        "[optimization]",
        "mode = 1",
        f"targets filename = {targets}",
        f"comparison mode = {comparison}",
        f"endo-epi minimization criterion epi delay = {endo_epi}",
        f"peak position is criterion = {peak}",
        f"optimize measuring points = {optimize_points}",
        "population size = 100",
        "number of generations = 100",
        f"fast approximation is criterion = {fast_is_crit}",
        f"fast approximation epi delay = {fast_delay}",
        f"fast approximation limit = {fast_limit}",
    ]
    if extra_opt:
        lines.append(extra_opt)
    return "\n".join(lines) + "\n"


def analytic_target(n_leads: int, steps: int, seed: int) -> np.ndarray:
    """Seeded smooth stand-in target (a few Gaussian bumps per lead) for workloads whose
    targets only feed the criteria reduction."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.arange(steps, dtype=np.float64)
    out = np.zeros((n_leads, steps))
    for l in range(n_leads):
        for _ in range(3):
            c, w, a = rng.uniform(0, steps), rng.uniform(10, 80), rng.uniform(-2, 2)
            out[l] += a * np.exp(-0.5 * ((t - c) / w) ** 2)
    return out


@dataclass
class Workload:
    """A heart plus its files on disk (directory ``root``)."""
    root: str
    spec: HeartSpec
    grid: np.ndarray
    transfer: np.ndarray
    leads_xyz: np.ndarray
    steps: int
    files: dict = field(default_factory=dict)


def make_workload(root: str, spec: HeartSpec, steps: int, target: Optional[np.ndarray] = None,
                  write_model: bool = True, **ini_kw) -> Workload:
    """Generate one heart and write model, conduction, points, ini and target into ``root``."""
    os.makedirs(root, exist_ok=True)
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    grid = ellipsoid_heart(spec)
    t = transfer_matrix(spec.n_layers, spec.delays)
    pts = leads(spec, rng)
    files = dict(shape="model.matrix", transfer="conduction.matrix", points="leads.txt",
                 targets="target.column", ini="simulator.ini")
    if write_model:
        write_matrix(os.path.join(root, files["shape"]), grid)
    write_transfer(os.path.join(root, files["transfer"]), t)
    write_points(os.path.join(root, files["points"]), pts)
    if target is None:
        target = analytic_target(spec.n_leads, steps, spec.seed + 999)
    write_column(os.path.join(root, files["targets"]), 0.0, 1.0, target)
    base = ini_kw.pop("base_aps", None) or tuple([BASE_AP] * max(3, min(spec.n_layers, 3)))
    with open(os.path.join(root, files["ini"]), "w") as f:
        f.write(ini_text(shape=files["shape"], transfer=files["transfer"], points=files["points"],
                         targets=files["targets"], length=steps, base_aps=base, **ini_kw))
    return Workload(root, spec, grid, t, pts, steps, files)


def genes_for(spec: HeartSpec, request: int, config_index: int = 0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(config_index * 1000 + request))
    return draw_genes(rng, spec.n_leads)
