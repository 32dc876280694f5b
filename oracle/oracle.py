"""FP64 CPU oracle for the EkgSim simulation path (TEST INFRASTRUCTURE ONLY).

Only the test suite, the smoke check and the benchmark's CPU-baseline leg use this module;
the engine in ``ekgsim_gb300`` never imports it.  It wraps ``ekg_oracle.c`` (an operation-for-
operation C restatement of the reference, see that file's header for file:line citations) and
restates the reference's file readers and evaluation driver in Python:

* ``.matrix`` reader: simlib/matrix.h:134-248 (importMatrix, shapeLoad :125-129)
* measuring points reader: simlib/simulator.cpp:369-397
* ``simulator.ini`` keys: simlib/simulator.h:107-145, SimSettings.h:158-356
* target loading and resampling: sim.cpp:999-1042, vectorMath.h:161-227
* evaluation driver: sim.cpp:443-492 (eval), :600-702 (calculateFitness), :712-747 (runApproxAndSim)
"""
from __future__ import annotations

import ctypes
import math
import os
import platform
import subprocess
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", platform.machine(), "libekg_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile ekg_oracle.c into oracle/_build/libekg_oracle.so (gcc, -ffp-contract=off)."""
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    src = os.path.join(_HERE, "ekg_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        tmp = _LIB_PATH + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        d, i32, i64 = ctypes.c_double, ctypes.c_int32, ctypes.c_int64
        L.ekgo_activation.argtypes = [ctypes.c_int] * 3 + [P(i32), ctypes.c_int, P(d), P(d), P(i32)]
        L.ekgo_run.argtypes = [ctypes.c_int] * 3 + [P(i32), P(d), ctypes.c_int, P(d), ctypes.c_int, P(d),
                                                    ctypes.c_int, d, d, d, P(d), ctypes.c_int]
        L.ekgo_run_naive.argtypes = [ctypes.c_int] * 3 + [P(i32), P(d), ctypes.c_int, P(d), ctypes.c_int, P(d),
                                                          ctypes.c_int, d, d, d, ctypes.c_int, P(d)]
        L.ekgo_run_naive_range.argtypes = [ctypes.c_int] * 3 + [P(i32), P(d), ctypes.c_int, P(d), ctypes.c_int,
                                                                P(d), ctypes.c_int, d, d, d, i64, i64, P(d)]
        L.ekgo_ap_indices.argtypes = [i64, P(i32), P(d), P(i64), P(i32), P(d)]
        L.ekgo_ap_indices.restype = i64
        L.ekgo_layer_aps.argtypes = [ctypes.c_int, ctypes.c_int, P(d), P(d), P(d), ctypes.c_uint,
                                     ctypes.c_int, d, P(d), P(d), P(d)]
        L.ekgo_move_leads.argtypes = [ctypes.c_int, P(d), P(d), P(d)]
        L.ekgo_compare.argtypes = [ctypes.c_int, P(d), i64, P(d), i64, d]
        L.ekgo_compare.restype = d
        L.ekgo_clamp.argtypes = [d]
        L.ekgo_clamp.restype = d
        L.ekgo_wohl.argtypes = [P(d), d]
        L.ekgo_wohl.restype = d
        L.ekgo_neighbourhood.argtypes = [ctypes.c_int, P(ctypes.c_int)]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


NHOOD = {"3D4": 0, "3D8": 1, "cube": 1, "2D4": 2, "2D8": 3}


# ------------------------------------------------------------------ kernels of the path
def activation(raw: np.ndarray, tm: np.ndarray):
    """Activation times (FP64) and stripped layers of a signed layer grid [z][y][x]."""
    raw = np.ascontiguousarray(raw, dtype=np.int32)
    tm = np.ascontiguousarray(tm, dtype=np.float64)
    nz, ny, nx = raw.shape
    at = np.zeros(raw.shape, dtype=np.float64)
    layer = np.zeros(raw.shape, dtype=np.int32)
    rc = lib().ekgo_activation(nz, ny, nx, _p(raw, ctypes.c_int32), tm.shape[0], _p(tm, ctypes.c_double),
                               _p(at, ctypes.c_double), _p(layer, ctypes.c_int32))
    if rc != 0:
        raise RuntimeError({-1: "Could not find starting point for excitation sequence",
                            -2: "transfer (conduction) matrix does not define layer"}.get(rc, f"oracle error {rc}"))
    return at, layer


def ap_indices(layer: np.ndarray, at: np.ndarray):
    layer = np.ascontiguousarray(layer, dtype=np.int32).ravel()
    at = np.ascontiguousarray(at, dtype=np.float64).ravel()
    n = layer.size
    idx = np.zeros(n, dtype=np.int64)
    al = np.zeros(n, dtype=np.int32)
    aa = np.zeros(n, dtype=np.float64)
    na = lib().ekgo_ap_indices(n, _p(layer, ctypes.c_int32), _p(at, ctypes.c_double), _p(idx, ctypes.c_int64),
                               _p(al, ctypes.c_int32), _p(aa, ctypes.c_double))
    return idx, al[:na].copy(), aa[:na].copy()


def run(layer: np.ndarray, at: np.ndarray, layer_k: np.ndarray, leads_zyx: np.ndarray, nhood="3D4",
        start=0.0, length=600.0, dt=1.0, threads=0) -> np.ndarray:
    """ECG [L, steps] in the reference's exact summation order."""
    layer = np.ascontiguousarray(layer, dtype=np.int32)
    at = np.ascontiguousarray(at, dtype=np.float64)
    layer_k = np.ascontiguousarray(layer_k, dtype=np.float64)
    leads_zyx = np.ascontiguousarray(np.atleast_2d(leads_zyx), dtype=np.float64)
    steps = int(math.ceil(length / dt))
    ecg = np.zeros((leads_zyx.shape[0], steps), dtype=np.float64)
    nz, ny, nx = layer.shape
    rc = lib().ekgo_run(nz, ny, nx, _p(layer, ctypes.c_int32), _p(at, ctypes.c_double), layer_k.shape[0],
                        _p(layer_k, ctypes.c_double), leads_zyx.shape[0], _p(leads_zyx, ctypes.c_double),
                        NHOOD[nhood], float(start), float(length), float(dt), _p(ecg, ctypes.c_double), threads)
    if rc != 0:
        raise RuntimeError(f"oracle run error {rc}")
    return ecg


def run_naive(layer, at, layer_k, leads_zyx, nhood="3D4", start=0.0, length=600.0, dt=1.0, steps_limit=0):
    """ECG with the reference's per-voxel AP evaluation cost (single thread), optionally only the
    first ``steps_limit`` steps."""
    layer = np.ascontiguousarray(layer, dtype=np.int32)
    at = np.ascontiguousarray(at, dtype=np.float64)
    layer_k = np.ascontiguousarray(layer_k, dtype=np.float64)
    leads_zyx = np.ascontiguousarray(np.atleast_2d(leads_zyx), dtype=np.float64)
    steps = int(math.ceil(length / dt))
    if 0 < steps_limit < steps:
        steps = steps_limit
    ecg = np.zeros((leads_zyx.shape[0], steps), dtype=np.float64)
    nz, ny, nx = layer.shape
    lib().ekgo_run_naive(nz, ny, nx, _p(layer, ctypes.c_int32), _p(at, ctypes.c_double), layer_k.shape[0],
                         _p(layer_k, ctypes.c_double), leads_zyx.shape[0], _p(leads_zyx, ctypes.c_double),
                         NHOOD[nhood], float(start), float(length), float(dt), int(steps_limit),
                         _p(ecg, ctypes.c_double))
    return ecg


def run_naive_range(layer, at, layer_k, leads_zyx, nhood="3D4", start=0.0, length=600.0, dt=1.0, k0=0, k1=None):
    """Steps [k0, k1) of the ECG with the reference's per-voxel cost structure (single thread); the
    values equal the same columns of run_naive over the whole axis."""
    layer = np.ascontiguousarray(layer, dtype=np.int32)
    at = np.ascontiguousarray(at, dtype=np.float64)
    layer_k = np.ascontiguousarray(layer_k, dtype=np.float64)
    leads_zyx = np.ascontiguousarray(np.atleast_2d(leads_zyx), dtype=np.float64)
    steps = int(math.ceil(length / dt))
    k1 = steps if k1 is None else min(int(k1), steps)
    ecg = np.zeros((leads_zyx.shape[0], max(0, k1 - int(k0))), dtype=np.float64)
    nz, ny, nx = layer.shape
    rc = lib().ekgo_run_naive_range(nz, ny, nx, _p(layer, ctypes.c_int32), _p(at, ctypes.c_double), layer_k.shape[0],
                                    _p(layer_k, ctypes.c_double), leads_zyx.shape[0], _p(leads_zyx, ctypes.c_double),
                                    NHOOD[nhood], float(start), float(length), float(dt), int(k0), int(k1),
                                    _p(ecg, ctypes.c_double))
    if rc != 0:
        raise RuntimeError(f"oracle run error {rc}")
    return ecg


def wohl(k, t: float) -> float:
    k = np.ascontiguousarray(k, dtype=np.float64)
    return lib().ekgo_wohl(_p(k, ctypes.c_double), float(t))


def layer_aps(n_layers: int, base: np.ndarray, kmin, kmax, free_k, interpolation: str, mid_position: float,
              genes: np.ndarray):
    base = np.ascontiguousarray(np.atleast_2d(base), dtype=np.float64)
    kmin = np.ascontiguousarray(kmin, dtype=np.float64)
    kmax = np.ascontiguousarray(kmax, dtype=np.float64)
    genes = np.ascontiguousarray(genes, dtype=np.float64)
    mask = 0
    for k in free_k:
        mask |= 1 << int(k)
    out = np.zeros((n_layers, 9), dtype=np.float64)
    viol = np.zeros(1, dtype=np.float64)
    interp = {"endo-epi": 1, "endo-mid-epi": 2}[interpolation]
    rc = lib().ekgo_layer_aps(n_layers, base.shape[0], _p(base, ctypes.c_double), _p(kmin, ctypes.c_double),
                              _p(kmax, ctypes.c_double), mask, interp, float(mid_position),
                              _p(genes, ctypes.c_double), _p(out, ctypes.c_double), _p(viol, ctypes.c_double))
    return out, float(viol[0]), int(rc)


def move_leads(orig_zyx: np.ndarray, disp: Optional[np.ndarray]) -> np.ndarray:
    orig = np.ascontiguousarray(np.atleast_2d(orig_zyx), dtype=np.float64)
    out = np.zeros_like(orig)
    if disp is None:
        lib().ekgo_move_leads(orig.shape[0], _p(orig, ctypes.c_double), None, _p(out, ctypes.c_double))
    else:
        dd = np.ascontiguousarray(disp, dtype=np.float64)
        lib().ekgo_move_leads(orig.shape[0], _p(orig, ctypes.c_double), _p(dd, ctypes.c_double),
                              _p(out, ctypes.c_double))
    return out


def compare(mode: int, a: np.ndarray, b: np.ndarray, bofs: float = 0.0) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().ekgo_compare(mode, _p(a, ctypes.c_double), a.size, _p(b, ctypes.c_double), b.size, float(bofs))


def clamp(c: float) -> float:
    return lib().ekgo_clamp(float(c))


# ------------------------------------------------------------------ file readers
def read_matrix(path: str, signed_layers: bool = True) -> np.ndarray:
    """importMatrix for the delimited forms ("space", "tab", "comma"); returns [z][y][x] (3d) or
    [y][x] (2d).  Character-coded files (no separator word) are read per character."""
    with open(path, "r") as f:
        f.readline()
        head = f.readline()
        body = f.read()
    parts = head.replace("x", " x ").split()
    dim = int(parts[0][0])
    sizes = [int(p) for p in parts[1:] if p.lstrip("-").isdigit()][:dim]
    sep = parts[-1] if not parts[-1].lstrip("-").isdigit() else ""
    shape = tuple(reversed(sizes))
    count = int(np.prod(shape))
    if sep in ("space", "tab", "comma", ","):
        txt = body.replace(",", " ")
        vals = np.array(txt.split()[:count], dtype=np.float64)
    else:
        chars = [c for c in body if not c.isspace()][:count]
        vals = []
        for ch in chars:
            if ch in "xX":
                vals.append(-1)
            elif ch >= "a":
                vals.append(ord(ch) - ord("a") + 10)
            elif ch >= "A":
                vals.append(ord(ch) - ord("A") + 10)
            else:
                vals.append(ord(ch) - ord("0"))
        vals = np.array(vals, dtype=np.float64)
    if vals.size != count:
        raise RuntimeError(f"reading file {path} failed (while reading data)")
    return vals.reshape(shape)


def read_points(path: str) -> np.ndarray:
    """Measuring points as (L, 3) in (z, y, x) order (the file holds x, y, z)."""
    pts = []
    with open(path) as f:
        for line in f:
            q = [s for s in line.replace(",", " ").split()]
            if len(q) < 3:
                break
            x, y, z = float(q[0]), float(q[1]), float(q[2])
            pts.append((z, y, x))
    return np.array(pts, dtype=np.float64)


def read_column(path: str) -> List[np.ndarray]:
    rows = []
    with open(path) as f:
        lines = f.read().splitlines()
    i = 0
    while i < len(lines) and lines[i][:1] in ("#", "%"):
        i += 1
    ncol = None
    for line in lines[i:]:
        vals = line.split()
        try:
            v = [float(s) for s in vals]
        except ValueError:
            break
        if ncol is None:
            ncol = len(v)
            if ncol == 0:
                raise RuntimeError("File has 0 columns")
        if len(v) < ncol:
            break
        rows.append(v[:ncol])
    arr = np.array(rows, dtype=np.float64)
    return [arr[:, c].copy() for c in range(arr.shape[1])]


def read_ini(path: str) -> Dict[str, Dict[str, str]]:
    out: Dict[str, Dict[str, str]] = {}
    sec = ""
    with open(path) as f:
        for raw in f:
            line = raw.split(";")[0].strip()
            if not line:
                continue
            if line.startswith("[") and "]" in line:
                sec = line[1:line.index("]")].strip()
                out.setdefault(sec, {})
                continue
            if "=" in line:
                k, v = line.split("=", 1)
                out.setdefault(sec, {})[k.strip()] = v.strip()
    return out


def _vec(s: str) -> List[float]:
    return [float(x) for x in s.replace(",", " ").split()]


def resample(src: np.ndarray, factor: float, start_offset: int) -> np.ndarray:
    """vectorMath.h:210-227 (factor == 1 copies the source and ignores the offset)."""
    if factor == 1:
        return src.copy()
    n = 1 + int(math.ceil((src.size - 1 - start_offset) * factor))
    dest = np.zeros(n)
    for i in range(n):
        old = i / factor + start_offset
        fp = int(math.floor(old))
        cp = int(1.0 + fp)
        if cp < src.size:
            dest[i] = src[cp] * (old - fp) + src[fp] * (cp - old)
        else:
            dest[i] = src[-1]
    return dest


def export_excitation(at: np.ndarray) -> str:
    """Text of an exported excitation sequence: exportShape with excit = true
    (simlib/simulator.cpp:71-106): a comment line, the "3D X x Y x Z tab" (or "2D X x Y tab")
    header, then per z block one line per y row of tab-separated times printed with three
    decimals, and an empty line after each block."""
    nz, ny, nx = at.shape
    out = ["Excitation file (next line specifies matrix type (2D) size (X x Y x Z) and elemet separator type "
           "(tab) after that comes data (x are rows, y are lines, z are blocks - separated with empty line)\n"]
    out.append(f"3D {nx} x {ny} x {nz} tab\n" if nz > 1 else f"2D {nx} x {ny} tab\n")
    for z in range(nz):
        for y in range(ny):
            out.append("\t".join("%.3f" % v for v in at[z, y]) + "\n")
        out.append("\n")
    return "".join(out)


def read_excitation(path: str, shape) -> np.ndarray:
    """Simulation::loadExcitationSequence (simlib/simulator.cpp:288-367) for a .matrix file: skip
    the comment line, read the "<d>D X x Y [x Z] <sep>" header, check the size against the shape,
    then read one time per cell in z, y, x order (stream extraction, a comma separator skipped)."""
    if not path.endswith(".matrix"):
        raise RuntimeError("can only import from .matrix for the time being")
    try:
        text = open(path).read()
    except OSError:
        raise RuntimeError(f"could not open file {path} to load excitation sequence")
    body = text.split("\n", 1)[1] if "\n" in text else ""
    toks = body.split(None, 1)
    dim = toks[0] if toks else ""
    if len(dim) < 2 or dim[1] not in "dD" or not ("0" < dim[0] <= "3"):
        raise RuntimeError("error while loading matrix, could not read dimensionality")
    rest = toks[1] if len(toks) > 1 else ""
    header, data = (rest.split("\n", 1) + [""])[:2]
    sizes = [int(v) for v in header.replace("x", " ").split()[:int(dim[0])]]
    size = [1, 1, 1]
    for i, v in enumerate(sizes):  # X first, then Y, then Z
        size[2 - i] = v
    if tuple(size) != tuple(shape):
        raise RuntimeError("failed to read excitation sequence due to its incompatible size")
    vals = np.array([float(v) for v in data.replace(",", " ").split()[: shape[0] * shape[1] * shape[2]]])
    if vals.size < shape[0] * shape[1] * shape[2]:
        vals = np.concatenate([vals, np.zeros(shape[0] * shape[1] * shape[2] - vals.size)])
    return vals.reshape(shape)


@dataclass
class Setup:
    """Everything SimImplementation's constructor loads (sim.cpp:362-431)."""
    raw: np.ndarray
    tm: np.ndarray
    leads_zyx: np.ndarray
    start: float
    length: float
    dt: float
    nhood: str
    interpolation: str
    mid: float
    base: np.ndarray
    kmin: np.ndarray
    kmax: np.ndarray
    free_k: List[int]
    optimize_points: bool
    comparison: int
    targets: List[np.ndarray]
    target_offsets: List[float]
    peak: bool = False
    endo_epi_delay: float = -1.0
    fast_is_crit: bool = False
    fast_delay: float = 0.0
    fast_limit: float = 2.0
    at: Optional[np.ndarray] = None
    layer: Optional[np.ndarray] = None
    n_layers: int = 0
    extra: dict = field(default_factory=dict)


def load_setup(workdir: str, ini_name: str = "simulator.ini") -> Setup:
    ini = read_ini(os.path.join(workdir, ini_name))
    m, sim, wa, opt = ini.get("model", {}), ini.get("simulation", {}), ini.get("wohlfart ap", {}), ini.get("optimization", {})
    raw = read_matrix(os.path.join(workdir, m["shape"])).astype(np.int32)
    if raw.ndim == 2:
        raw = raw[None]
    tm = read_matrix(os.path.join(workdir, m["transfer"]))
    pts = read_points(os.path.join(workdir, m["points"]))
    base = []
    i = 1
    while f"base ap {i}" in wa:
        v = _vec(wa[f"base ap {i}"])[:9]
        if len(v) != 9:
            break
        base.append(v)
        i += 1
    mid = float(wa.get("mid AP position", 0.5))
    if mid > 1.0 or mid < 0.0:
        mid = 0.5
    start = float(int(float(sim.get("start", 0))))
    length = float(int(float(sim.get("length", 800))))
    dt = float(sim.get("time step", 1.0 / 3.0))
    # targets (sim.cpp:999-1042)
    cols = read_column(os.path.join(workdir, opt["targets filename"]))
    ntarg = max(1, len(cols) - 1)
    target_dt = 1.0
    ecg_cols = min(1, len(cols) - 1)
    if ecg_cols > 0:
        target_dt = cols[0][1] - cols[0][0]
    rstart = int(start / target_dt)
    targets, offsets = [None] * ntarg, [0.0] * ntarg
    for c in range(ecg_cols, len(cols)):
        col = cols[c].copy()
        tmin, tmax = col[0], col[0]
        for v in col[1:]:
            if v < tmin:
                tmin = v
            elif v > tmax:
                tmax = v
        col = col * (1.0 / (tmax - tmin))
        targets[c - ecg_cols] = resample(col, target_dt / dt, rstart)
        offsets[c - ecg_cols] = 1.0 - (tmin / (tmax - tmin))
    s = Setup(raw=raw, tm=tm, leads_zyx=pts, start=start, length=length, dt=dt,
              nhood=sim.get("neighbourhood type", "3D4"), interpolation=wa.get("interpolation", ""), mid=mid,
              base=np.array(base), kmin=np.array(_vec(wa["k min"])), kmax=np.array(_vec(wa["k max"])),
              free_k=[int(x) for x in _vec(wa.get("free k", ""))],
              optimize_points=bool(int(float(opt.get("optimize measuring points", 0)))),
              comparison=int(float(opt.get("comparison mode", 2))), targets=targets, target_offsets=offsets,
              peak=int(float(opt.get("peak position is criterion", 0))) > 0,
              endo_epi_delay=float(opt.get("endo-epi minimization criterion epi delay", -1)),
              fast_is_crit=int(float(opt.get("fast approximation is criterion", 0))) > 0,
              fast_delay=float(opt.get("fast approximation epi delay", 0)),
              fast_limit=float(opt.get("fast approximation limit", 2)))
    ex_in = m.get("excitation sequence", "")
    if ex_in:
        # simlib/sim_lib.h:224-231: a precomputed sequence replaces the cellular automaton
        s.layer = np.abs(s.raw).astype(np.int32)
        s.at = read_excitation(os.path.join(workdir, ex_in), s.raw.shape)
    else:
        s.at, s.layer = activation(s.raw, s.tm)
    s.n_layers = int(s.layer.max())
    return s


def evaluate(s: Setup, genes: np.ndarray, threads: int = 0):
    """OptimizationFunction::operator() for criteria mode 1 (sim.cpp:443-492, :600-702).
    Returns (criteria, violation, ecg [L, steps], layer_k, moved leads (z,y,x))."""
    genes = np.asarray(genes, dtype=np.float64)
    nfree = len(set(s.free_k))
    n_w = nfree * (3 if s.interpolation == "endo-mid-epi" else 2)
    n_d = 2 * s.leads_zyx.shape[0] if s.optimize_points else 0
    if genes.size != n_w + n_d:
        raise RuntimeError("chromosome size does not agree with the combination of the number of free "
                           "Wohlfart parameters and the selected interpolation procedure")
    leads = s.leads_zyx
    if s.optimize_points:
        leads = move_leads(s.leads_zyx, genes[n_w:].reshape(-1, 2))
    lk, viol, _ = layer_aps(s.n_layers, s.base, s.kmin, s.kmax, sorted(set(s.free_k)), s.interpolation, s.mid,
                            genes[:n_w])
    steps = int(math.ceil(s.length / s.dt))
    # fast approximation gate (sim.cpp:712-747, simlib/simulator.cpp:552-559)
    approx_crit = 2.0
    approx = None
    if s.fast_is_crit or s.fast_limit < 2:
        n = int(s.length / s.dt)
        approx = np.array([wohl(lk[0], (s.start + i * s.dt) + s.fast_delay) - wohl(lk[-1], s.start + i * s.dt)
                           for i in range(n)])
        approx_crit = compare(s.comparison, approx, s.targets[0], s.target_offsets[0])
    done = not (approx_crit > s.fast_limit)
    ecg = run(s.layer, s.at, lk, leads, s.nhood, s.start, s.length, s.dt, threads) if done else None
    nm = min(leads.shape[0], len(s.targets))
    ncrit = nm + (nm if s.peak else 0) + (1 if s.fast_is_crit else 0) + (1 if s.endo_epi_delay >= 0 else 0)
    res = np.zeros(ncrit)
    if s.fast_is_crit:
        res[nm] = approx_crit
    for i in range(nm):
        if done:
            simr = ecg[i]
            c = compare(s.comparison, simr, s.targets[i], s.target_offsets[i])
        else:
            simr = approx
            c = approx_crit
        ci = i
        if s.peak:
            ci = 2 * i
            res[ci + 1] = abs(int(np.argmax(simr)) - int(np.argmax(s.targets[i])))
        res[ci] = clamp(c)
    if s.endo_epi_delay >= 0:
        sd = 0.0
        t = 1.0
        while t < 700.0:
            d = wohl(lk[0], t + s.endo_epi_delay) - wohl(lk[-1], t)
            sd += d * d
            t += 1.0
        res[-1] = sd
    return res, viol, ecg, lk, leads
