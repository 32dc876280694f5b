"""Python handles over the C ABI: Engine, Heart and Server.

These wrap include/ekgsim.h one to one; numpy arrays cross the boundary as plain pointers.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib as L
from ._lib import EkgError, check, dptr, i32ptr, i64ptr  # noqa: F401 (EkgError is part of this module's API)


class Engine:
    """One engine per process and GPU (ekg_engine_create)."""

    def __init__(self, device: int = 0):
        self._lib = L.load()
        h = ctypes.c_void_p()
        check(self._lib.ekg_engine_create(device, ctypes.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def free_bytes(self) -> int:
        v = ctypes.c_uint64()
        check(self._lib.ekg_engine_free_bytes(self._h, ctypes.byref(v)))
        return int(v.value)

    def close(self):
        if self._h:
            check(self._lib.ekg_engine_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Heart:
    """A resident heart: activation times, de-duplicated APs and lead field live on the device."""

    def __init__(self, engine: Engine, handle):
        self.engine = engine
        self._lib = engine._lib
        self._h = handle
        self.info = self._info()

    @classmethod
    def create(cls, engine: Engine, layers: np.ndarray, transfer: np.ndarray, leads_zyx: np.ndarray,
               nhood: str = "3D4", start: float = 0.0, length: float = 600.0, dt: float = 1.0,
               activation: Optional[np.ndarray] = None) -> "Heart":
        """Upload a heart.  `activation` (same shape as `layers`) replaces the computed activation
        times, as a loaded excitation sequence does in the reference."""
        layers = np.ascontiguousarray(layers, dtype=np.int32)
        if layers.ndim == 2:
            layers = layers[None]
        transfer = np.ascontiguousarray(transfer, dtype=np.float64)
        leads_zyx = np.ascontiguousarray(np.atleast_2d(leads_zyx), dtype=np.float64)
        at_in = None
        if activation is not None:
            at_in = np.ascontiguousarray(activation, dtype=np.float64).reshape(layers.shape)
        d = L.HeartDesc(layers.shape[0], layers.shape[1], layers.shape[2], i32ptr(layers), transfer.shape[0],
                        dptr(transfer), leads_zyx.shape[0], dptr(leads_zyx), L.NHOOD[nhood], float(start),
                        float(length), float(dt), dptr(at_in) if at_in is not None else None)
        h = ctypes.c_void_p()
        check(engine._lib.ekg_heart_create(engine.handle, ctypes.byref(d), ctypes.byref(h)))
        heart = cls(engine, h)
        heart.shape = layers.shape
        return heart

    @classmethod
    def from_ini(cls, engine: Engine, ini_path: str, out_dir: Optional[str] = None) -> "Heart":
        h = ctypes.c_void_p()
        check(engine._lib.ekg_heart_from_ini(engine.handle, ini_path.encode(),
                                             out_dir.encode() if out_dir else None, ctypes.byref(h)))
        heart = cls(engine, h)
        heart.shape = None
        return heart

    def _info(self) -> L.HeartInfo:
        i = L.HeartInfo()
        check(self._lib.ekg_heart_get_info(self._h, ctypes.byref(i)))
        return i

    @property
    def handle(self):
        return self._h

    @property
    def n_leads(self) -> int:
        return self.info.n_leads

    @property
    def steps(self) -> int:
        return self.info.steps

    def activation(self) -> np.ndarray:
        out = np.zeros(self.info.n_cells, dtype=np.float64)
        check(self._lib.ekg_heart_activation(self._h, dptr(out)))
        return out.reshape(self.shape) if self.shape is not None else out

    def ap_index(self) -> np.ndarray:
        out = np.zeros(self.info.n_cells, dtype=np.int64)
        check(self._lib.ekg_heart_ap_index(self._h, i64ptr(out)))
        return out.reshape(self.shape) if self.shape is not None else out

    def simulate(self, layer_k: np.ndarray, leads_zyx: Optional[np.ndarray] = None) -> np.ndarray:
        """ECG [n_leads, steps] for the given layer APs (and optionally moved leads)."""
        layer_k = np.ascontiguousarray(layer_k, dtype=np.float64)
        if layer_k.shape != (self.info.n_layers, 9):
            raise ValueError(f"layer_k must be ({self.info.n_layers}, 9)")
        lp = None
        if leads_zyx is not None:
            lp = np.ascontiguousarray(leads_zyx, dtype=np.float64)
            if lp.shape != (self.n_leads, 3):
                raise ValueError(f"leads must be ({self.n_leads}, 3)")
        out = np.zeros((self.n_leads, self.steps), dtype=np.float64)
        check(self._lib.ekg_simulate(self._h, dptr(layer_k), dptr(lp), dptr(out)))
        return out

    def benchmark(self, layer_k: np.ndarray, leads_zyx: Optional[np.ndarray] = None, warmup: int = 3,
                  iters: int = 10) -> dict:
        """Device-only timing with resident inputs (ekg_heart_benchmark)."""
        lk = np.ascontiguousarray(layer_k, dtype=np.float64)
        n = lk.shape[0] if lk.ndim == 3 else 1
        lp = None if leads_zyx is None else np.ascontiguousarray(leads_zyx, dtype=np.float64)
        out = np.zeros(11)
        check(self._lib.ekg_heart_benchmark(self._h, n, dptr(lk), dptr(lp), warmup, iters, dptr(out), 11))
        return dict(total_ms=out[0], contract_ms=out[1], prep_ms=out[2], tail_ms=out[3], launches=int(out[4]),
                    moved_leads=int(out[5]), batched=bool(out[6]), operand_ms=out[7], gemm_flops=out[8],
                    operand_bytes=out[9], band_bytes=out[10], iters=iters, n_sims=n)

    # ------------------------------------------------------------------ evaluation
    def tune(self, layer_k: np.ndarray, leads_zyx: Optional[np.ndarray] = None, reps: int = 3) -> dict:
        """Autotune the batched form's launch shapes for passes like this one (ekg_heart_tune)."""
        lk = np.ascontiguousarray(layer_k, dtype=np.float64)
        n = lk.shape[0]
        ld = None if leads_zyx is None else np.ascontiguousarray(leads_zyx, dtype=np.float64)
        out = np.zeros(7 + 5 * 64)
        check(self._lib.ekg_heart_tune(self._h, n, dptr(lk), dptr(ld), reps, dptr(out), out.size))
        nc = int(out[5])
        table = [{"tile_rows": int(out[7 + 5 * i]), "ctas_per_sm": int(out[8 + 5 * i]),
                  "operand_form": "per-(AP, simulation)" if out[9 + 5 * i] == 1 else "persistent",
                  "operand_blocks_per_sm": int(out[10 + 5 * i]), "ms": float(out[11 + 5 * i])}
                 for i in range(min(nc, 64))]
        return {"tile_rows": int(out[0]), "ctas_per_sm": int(out[1]), "operand_form":
                "per-(AP, simulation)" if out[2] == 1 else "persistent", "operand_blocks_per_sm": int(out[6]),
                "ms": float(out[3]), "builtin_ms": float(out[4]), "candidates": nc, "timings": table}

    def set_eval(self, base_aps, k_min, k_max, free_k, targets, target_offsets=None, **kw):
        """Evaluation settings (ekg_heart_set_eval); keyword arguments as ``eval_config``."""
        self._cfg = eval_config(base_aps, k_min, k_max, free_k, targets, target_offsets, **kw)
        self.eval_args = ((base_aps, k_min, k_max, free_k, targets, target_offsets), dict(kw))
        self._eval_shape = None
        check(self._lib.ekg_heart_set_eval(self._h, ctypes.byref(self._cfg)))

    def eval_shape(self):
        """(genes, criteria) per evaluation; kept until the evaluation settings change."""
        if getattr(self, "_eval_shape", None) is None:
            g, c = ctypes.c_int32(), ctypes.c_int32()
            check(self._lib.ekg_eval_shape(self._h, ctypes.byref(g), ctypes.byref(c)))
            self._eval_shape = (g.value, c.value)
        return self._eval_shape

    def gene_bounds(self):
        g, _ = self.eval_shape()
        lo, hi = np.zeros(g), np.zeros(g)
        check(self._lib.ekg_eval_gene_bounds(self._h, dptr(lo), dptr(hi)))
        return lo, hi

    def eval(self, genes, want_ecg: bool = False):
        """One evaluation: (criteria, violation[, ecg, layer_k, leads])."""
        genes = np.ascontiguousarray(genes, dtype=np.float64)
        ng, nc = self.eval_shape()
        crit = np.zeros(nc)
        viol = np.zeros(1)
        ecg = np.zeros((self.n_leads, self.steps)) if want_ecg else None
        lk = np.zeros((self.info.n_layers, 9)) if want_ecg else None
        leads = np.zeros((self.n_leads, 3)) if want_ecg else None
        check(self._lib.ekg_eval(self._h, dptr(genes), genes.size, dptr(crit), dptr(viol), dptr(ecg), dptr(lk),
                                 dptr(leads)))
        if want_ecg:
            return crit, float(viol[0]), ecg, lk, leads
        return crit, float(viol[0])

    def simulation_done(self) -> bool:
        """Whether the last eval() ran its simulation (False when the fast-approximation gate
        skipped it; ekg_eval_simulated)."""
        v = ctypes.c_int32(1)
        check(self._lib.ekg_eval_simulated(self._h, ctypes.byref(v)))
        return bool(v.value)

    def _batch_args(self, genes, want_ecg, out):
        genes = np.ascontiguousarray(np.atleast_2d(genes), dtype=np.float64)
        n, g = genes.shape
        _, nc = self.eval_shape()
        shapes = [(n, nc), (n,)] + ([(n, self.n_leads, self.steps)] if want_ecg else [])
        if out is not None:
            if len(out) != len(shapes) or any(
                    a.shape != sh or a.dtype != np.float64 or not a.flags.c_contiguous for a, sh in zip(out, shapes)):
                raise ValueError(f"out must be C-contiguous float64 arrays of shapes {shapes}")
            bufs = list(out)
        else:
            bufs = [np.empty(sh) for sh in shapes]
        return genes, n, g, bufs

    def eval_batch(self, genes: np.ndarray, want_ecg: bool = False, out=None):
        """Criteria [n, n_criteria], violations [n] (and ECGs [n, n_leads, steps]) for n gene vectors.
        ``out`` = (crit, viol[, ecg]) reuses caller-owned C-contiguous float64 arrays of those shapes."""
        genes, n, g, bufs = self._batch_args(genes, want_ecg, out)
        crit, viol = bufs[0], bufs[1]
        ecg = bufs[2] if want_ecg else None
        check(self._lib.ekg_eval_batch(self._h, n, genes.ctypes.data, g, crit.ctypes.data, viol.ctypes.data,
                                       ecg.ctypes.data if ecg is not None else None))
        return (crit, viol, ecg) if want_ecg else (crit, viol)

    def eval_batch_submit(self, genes: np.ndarray, out, want_ecg: bool = False) -> int:
        """Queues a batched evaluation into caller-owned ``out`` = (crit, viol[, ecg]) and returns its
        ticket; the arrays are complete after ``eval_batch_wait(ticket)`` (ekg_eval_batch_submit)."""
        genes, n, g, bufs = self._batch_args(genes, want_ecg, out)
        crit, viol = bufs[0], bufs[1]
        ecg = bufs[2] if want_ecg else None
        t = ctypes.c_int64()
        check(self._lib.ekg_eval_batch_submit(self._h, n, genes.ctypes.data, g, crit.ctypes.data, viol.ctypes.data,
                                              ecg.ctypes.data if ecg is not None else None, ctypes.byref(t)))
        return t.value

    def eval_batch_wait(self, ticket: int):
        check(self._lib.ekg_eval_batch_wait(self._h, ticket))

    def close(self):
        if self._h:
            check(self._lib.ekg_heart_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eval_config(base_aps, k_min, k_max, free_k, targets=(np.zeros(1),), target_offsets=None,
                interpolation="endo-mid-epi", mid_position=0.5, optimize_points=True, comparison_mode=2,
                criteria_mode=1, peak=False, fast_is_criterion=False, fast_delay=0.0, fast_limit=2.0,
                endo_epi_delay=-1.0, disp_min=(-50,), disp_max=(50,)):
    """An ekg_eval_config plus the arrays it points into (kept alive in ``cfg._keep``)."""
    keep = dict(
        base=np.ascontiguousarray(np.atleast_2d(base_aps), dtype=np.float64),
        kmin=np.ascontiguousarray(k_min, dtype=np.float64), kmax=np.ascontiguousarray(k_max, dtype=np.float64),
        tl=np.array([len(t) for t in targets], dtype=np.int64),
        tg=np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=np.float64) for t in targets])),
        to=np.ascontiguousarray(target_offsets if target_offsets is not None else np.zeros(len(targets)),
                                dtype=np.float64),
        dmin=np.ascontiguousarray(disp_min, dtype=np.float64), dmax=np.ascontiguousarray(disp_max, dtype=np.float64))
    mask = 0
    for f in free_k:
        mask |= 1 << int(f)
    k = keep
    c = L.EvalConfig(1 if interpolation == "endo-epi" else 2, mid_position, k["base"].shape[0], dptr(k["base"]),
                     dptr(k["kmin"]), dptr(k["kmax"]), mask, int(optimize_points), criteria_mode, comparison_mode,
                     int(peak), int(fast_is_criterion), fast_delay, fast_limit, endo_epi_delay, len(targets),
                     i64ptr(k["tl"]), dptr(k["tg"]), dptr(k["to"]), len(k["dmin"]), dptr(k["dmin"]),
                     len(k["dmax"]), dptr(k["dmax"]))
    c._keep = keep
    return c


def layer_aps(cfg, n_layers: int, wohlfart_genes) -> tuple:
    """Layer APs [n_layers, 9] and violation from the Wohlfart genes (host only)."""
    lib = L.load()
    g = np.ascontiguousarray(wohlfart_genes, dtype=np.float64)
    out = np.zeros((n_layers, 9))
    v = np.zeros(1)
    check(lib.ekg_layer_aps(ctypes.byref(cfg), n_layers, dptr(g), dptr(out), dptr(v)))
    return out, float(v[0])


def move_leads(orig_zyx: np.ndarray, disp_uv: Optional[np.ndarray]) -> np.ndarray:
    lib = L.load()
    o = np.ascontiguousarray(np.atleast_2d(orig_zyx), dtype=np.float64)
    out = np.zeros_like(o)
    d = None if disp_uv is None else np.ascontiguousarray(disp_uv, dtype=np.float64)
    check(lib.ekg_move_leads(o.shape[0], dptr(o), dptr(d), dptr(out)))
    return out


class Server:
    """Served form: request loop with continuous batching over resident hearts."""

    def __init__(self, engine: Engine, max_batch: int = 256, max_wait_us: int = 200, hbm_reserve_bytes: int = 2 << 30,
                 keep_ecg: bool = True):
        self.engine = engine
        self._lib = engine._lib
        o = L.ServerOpts(max_batch, max_wait_us, hbm_reserve_bytes, 0 if keep_ecg else 1)
        h = ctypes.c_void_p()
        check(self._lib.ekg_server_create(engine.handle, ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._hearts = {}

    def add_heart(self, heart: Heart) -> int:
        i = ctypes.c_int32()
        check(self._lib.ekg_server_add_heart(self._h, heart.handle, ctypes.byref(i)))
        self._hearts[i.value] = heart
        return i.value

    def submit(self, heart_id: int, genes) -> int:
        g = np.ascontiguousarray(genes, dtype=np.float64)
        rid = ctypes.c_uint64()
        check(self._lib.ekg_server_submit(self._h, heart_id, dptr(g), g.size, ctypes.byref(rid)))
        return rid.value

    def poll(self, request_id: int, heart_id: int, wait_ms: int = 0, want_ecg: bool = False):
        """(criteria, violation, ecg or None, stats dict) or None when not ready."""
        heart = self._hearts[heart_id]
        _, nc = heart.eval_shape()
        crit = np.zeros(nc)
        viol = np.zeros(1)
        ecg = np.zeros((heart.n_leads, heart.steps)) if want_ecg else None
        st = L.RequestStats()
        rc = self._lib.ekg_server_poll(self._h, request_id, wait_ms, dptr(crit), dptr(viol), dptr(ecg),
                                       ctypes.byref(st))
        if rc == -10:
            return None
        check(rc)
        return crit, float(viol[0]), ecg, dict(queue_ms=st.queue_ms, total_ms=st.total_ms, batch=st.batch_size)

    def submit_many(self, heart_ids, genes) -> np.ndarray:
        """Submit len(heart_ids) requests (genes: one row per request); returns their ids."""
        hid = np.ascontiguousarray(heart_ids, dtype=np.int32)
        g = np.ascontiguousarray(np.atleast_2d(genes), dtype=np.float64)
        ids = np.zeros(hid.size, dtype=np.uint64)
        check(self._lib.ekg_server_submit_many(self._h, hid.size, hid.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                               dptr(g), g.shape[1], ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        return ids

    def poll_many(self, ids, n_criteria: int, wait_ms: int = 0):
        """Hand over finished requests: (status [n], criteria [n, n_criteria], violation [n],
        total_ms [n], batch [n]); status -10 marks a request that is not finished yet."""
        ids = np.ascontiguousarray(ids, dtype=np.uint64)
        n = ids.size
        crit = np.zeros((n, n_criteria))
        viol = np.zeros(n)
        status = np.zeros(n, dtype=np.int32)
        stats = (L.RequestStats * max(1, n))()
        rc = self._lib.ekg_server_poll_many(self._h, n, ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), wait_ms,
                                            n_criteria, dptr(crit), dptr(viol),
                                            status.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), stats)
        if rc not in (0, -10):
            check(rc)
        total = np.array([stats[i].total_ms for i in range(n)])
        batch = np.array([stats[i].batch_size for i in range(n)])
        return status, crit, viol, total, batch

    def close(self):
        if self._h:
            check(self._lib.ekg_server_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def host_register(a: np.ndarray):
    """Page-locks a numpy array's memory (ekg_host_register) so device copies into it run asynchronously."""
    check(L.load().ekg_host_register(a.ctypes.data, a.nbytes))


def host_unregister(a: np.ndarray):
    check(L.load().ekg_host_unregister(a.ctypes.data))
