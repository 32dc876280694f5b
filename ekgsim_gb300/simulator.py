"""Python mirror of the reference's simulator interfaces, over the C ABI.

* ``EkgSim`` follows ``SimLib::EkgSim`` (simlib/sim_lib.h:78-287): load settings and model,
  simulate the excitation sequence, set layer APs, run, read measurements, save result.column.
* ``OptimizationFunction`` follows the evaluation hook AMS-DEMO calls (sim.h:97-123,
  AMS-DEMO/GeneralOptimizationAlgorithm.h:83-93): ``__call__(solution) -> (result, violation)``
  plus ``get_gene_params``, ``get_evolutionary_params`` and ``normalize``; ``evaluate_batch``
  runs a whole generation in one device pass.

Errors raise ``EkgError`` with the reference's messages.
"""
from __future__ import annotations

import os
from typing import List, Optional, Sequence

import numpy as np

from . import engine as E
from .engine import EkgError  # noqa: F401

_ENGINE: Optional[E.Engine] = None


def default_engine() -> E.Engine:
    global _ENGINE
    if _ENGINE is None:
        _ENGINE = E.Engine(0)
    return _ENGINE


class EkgSim:
    """loadSettings -> (loadShape, loadTransferMatrix, loadMeasuringPoints, simExcitationSequence,
    applySettings) -> setApsDestructive -> run -> getMeasurement, as in simlib/sim_lib.h:78-92."""

    def __init__(self, engine: Optional[E.Engine] = None):
        self.engine = engine or default_engine()
        self.heart: Optional[E.Heart] = None
        self._ini = None
        self._aps = None
        self._leads = None
        self._ecg = None

    # settings + model in one step (the ini names every file)
    def loadSettings(self, fname: str = "settings.ini"):
        self._ini = os.path.abspath(fname)

    def simExcitationSequence(self):
        if self._ini is None:
            raise EkgError(-1, "settings not loaded")
        self.heart = E.Heart.from_ini(self.engine, self._ini)

    def requiredAps(self) -> int:
        return self.heart.info.n_layers

    def setApsDestructive(self, layer_k: Sequence[Sequence[float]]):
        self._aps = np.array(layer_k, dtype=np.float64)

    def moveMeasuringPoints(self, uv_displacement: np.ndarray, original_zyx: np.ndarray):
        self._leads = E.move_leads(original_zyx, uv_displacement)

    def run(self):
        self._ecg = self.heart.simulate(self._aps, self._leads)

    def numMeasurements(self) -> int:
        return self.heart.n_leads

    def getMeasurement(self, n: int) -> np.ndarray:
        return self._ecg[n]

    def activationTimes(self) -> np.ndarray:
        return self.heart.activation()


class OptimizationFunction:
    """The AMS-DEMO evaluation hook for one simulator.ini (sim.cpp:1084-1129)."""

    def __init__(self, ini: str = "simulator.ini", engine: Optional[E.Engine] = None, out_dir: Optional[str] = "."):
        self.engine = engine or default_engine()
        self.heart = E.Heart.from_ini(self.engine, ini, out_dir)
        self.num_genes, self.num_criteria = self.heart.eval_shape()
        self.gene_min, self.gene_max = self.heart.gene_bounds()

    def __call__(self, solution: Sequence[float]):
        crit, viol = self.heart.eval(np.asarray(solution, dtype=np.float64))
        return list(crit), viol

    def simulation_done(self) -> bool:
        """SimImplementation::simulationDone (sim.cpp:712-748) for the last call."""
        return self.heart.simulation_done()

    def evaluate_batch(self, solutions: np.ndarray):
        crit, viol = self.heart.eval_batch(np.asarray(solutions, dtype=np.float64))
        return crit, viol

    def get_gene_params(self):
        return self.num_genes, self.num_criteria, list(self.gene_min), list(self.gene_max)

    def normalize(self, solution: List[float]) -> List[float]:
        s = list(solution)
        for i in range(min(len(s), len(self.gene_min))):
            s[i] = max(s[i], self.gene_min[i])
        for i in range(min(len(s), len(self.gene_max))):
            s[i] = min(s[i], self.gene_max[i])
        return s
