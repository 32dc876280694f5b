"""The allocation-free activation entry point (ekg_activation_noalloc).

It serves callers that cannot call cudaMalloc -- code running under a framework's memory pool or
in a loop that must not allocate device memory.  The caller owns the input and output device
buffers (here torch tensors stand in for them); the entry point's own scratch is a fixed array
inside the library.  Its output must match the regular heart set-up bit for bit, on two calls in
a row with different hearts (the shared scratch must not carry stale state between calls).
This file sorts last so that a failing run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from ekgsim_gb300 import synth

pytestmark = pytest.mark.gpu


def _noalloc(grid, tm):
    torch = pytest.importorskip("torch")
    from ekgsim_gb300 import _lib as L
    lib = L.load()
    dev_layers = torch.from_numpy(np.ascontiguousarray(grid, dtype=np.int32)).cuda()
    dev_at = torch.full(grid.shape, -7.0, dtype=torch.float64, device="cuda")  # stale content on purpose
    tmc = np.ascontiguousarray(tm, dtype=np.float64)
    rounds = ctypes.c_int32(0)
    torch.cuda.synchronize()
    nz, ny, nx = grid.shape
    rc = lib.ekg_activation_noalloc(nz, ny, nx, ctypes.c_void_p(dev_layers.data_ptr()), tmc.shape[0], L.dptr(tmc),
                                    ctypes.c_void_p(dev_at.data_ptr()), ctypes.byref(rounds))
    L.check(rc)
    return dev_at.cpu().numpy(), rounds.value


def _regular(grid, tm):
    from ekgsim_gb300.engine import Engine, Heart
    eng = Engine(0)
    h = Heart.create(eng, grid, tm, np.array([[0.0, 0.0, 200.0]]), "3D4", 0.0, 10.0, 1.0)
    at = h.activation()
    h.close()
    eng.close()
    return at


def test_noalloc_matches_regular_twice():
    specs = [synth.small_spec(24), synth.config(0)["spec"]]
    for spec in specs:  # two calls in a row, different sizes
        grid = synth.ellipsoid_heart(spec)
        tm = synth.transfer_matrix(spec.n_layers, spec.delays)
        at_na, rounds = _noalloc(grid, tm)
        at_reg = _regular(grid, tm)
        assert rounds > 0
        assert np.array_equal(at_na.view(np.int64), at_reg.view(np.int64))
    # the smaller heart again after the larger one
    grid = synth.ellipsoid_heart(specs[0])
    tm = synth.transfer_matrix(3, specs[0].delays)
    at_na, _ = _noalloc(grid, tm)
    assert np.array_equal(at_na.view(np.int64), _regular(grid, tm).view(np.int64))


def test_noalloc_rejects_oversized_grid():
    torch = pytest.importorskip("torch")
    from ekgsim_gb300 import _lib as L
    lib = L.load()
    tm = np.ascontiguousarray(synth.transfer_matrix(3, [1, 2, 2]))
    dummy = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = lib.ekg_activation_noalloc(512, 512, 512, ctypes.c_void_p(dummy.data_ptr()), tm.shape[0], L.dptr(tm),
                                    ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -1
    assert b"65536 tiles" in lib.ekg_last_error()
