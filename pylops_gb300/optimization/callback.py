"""Solver callbacks (``pylops/optimization/callback.py:16-183``)."""

import numpy as np

from ..utils.backend import to_numpy

__all__ = ["Callbacks", "MetricsCallback"]


class Callbacks:
    """Template: subclass and override the ``on_*`` hooks; each receives the
    solver and the current model vector."""

    def on_setup_begin(self, solver, x0):
        pass

    def on_setup_end(self, solver, x):
        pass

    def on_step_begin(self, solver, x):
        pass

    def on_step_end(self, solver, x):
        pass

    def on_run_begin(self, solver, x):
        pass

    def on_run_end(self, solver, x):
        pass


class MetricsCallback(Callbacks):
    """Store mae/mse/snr/psnr of the iterates against a true model
    (``callback.py:115-183``)."""

    def __init__(self, xtrue, Op=None, which=("mae", "mse", "snr", "psnr")):
        self.xtrue = to_numpy(xtrue).ravel()
        self.Op = Op
        self.which = which
        self.metrics = {k: [] for k in which}

    def on_step_end(self, solver, x):
        xe = to_numpy(x).ravel().astype(np.float64)
        xt = self.xtrue.astype(np.float64)
        err = xe - xt
        mse = float(np.mean(err ** 2))
        if "mae" in self.which:
            self.metrics["mae"].append(float(np.mean(np.abs(err))))
        if "mse" in self.which:
            self.metrics["mse"].append(mse)
        if "snr" in self.which:
            self.metrics["snr"].append(float(10 * np.log10(np.sum(xt ** 2) / max(np.sum(err ** 2), 1e-300))))
        if "psnr" in self.which:
            self.metrics["psnr"].append(float(10 * np.log10(np.max(np.abs(xt)) ** 2 / max(mse, 1e-300))))
