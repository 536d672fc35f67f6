"""Solver template (``pylops/optimization/basesolver.py:18-330``)."""

import functools
import time
from abc import ABCMeta, abstractmethod

__all__ = ["Solver"]

_units = {"B": 1, "KB": 1024, "MB": 1024 ** 2, "GB": 1024 ** 3}


class Solver(metaclass=ABCMeta):
    """Base class with the setup/step/run/finalize/solve life cycle and
    callback decoration of the reference (``basesolver.py:56-120``)."""

    def __init__(self, Op, callbacks=None) -> None:
        self.Op = Op
        self.callbacks = callbacks
        self._registercallbacks()
        self.iiter = 0
        self.tstart = time.time()

    def _print_solver(self, text: str = "", nbar: int = 80) -> None:
        print(f"{type(self).__name__}" + text)
        print("-" * nbar + "\n" f"The Operator Op has {self.Op.shape[0]} rows and {self.Op.shape[1]} cols")

    def _print_setup(self, *args, **kwargs) -> None:
        pass

    def _print_step(self, *args, **kwargs) -> None:
        pass

    def _print_finalize(self, *args, nbar: int = 80, **kwargs) -> None:
        print(f"\nIterations = {self.iiter}        Total time (s) = {self.telapsed:.2f}")
        print("-" * nbar + "\n")

    def _registercallbacks(self) -> None:
        def cbdecorator(func, setup=False):
            @functools.wraps(func)
            def wrapper(*args, **kwargs):
                if self.callbacks:
                    for cb in self.callbacks:
                        x = kwargs.get("x0", None) if setup else args[0]
                        getattr(cb, f"on_{func.__name__}_begin")(self, x)
                ret = func(*args, **kwargs)
                if self.callbacks:
                    for cb in self.callbacks[::-1]:
                        x = kwargs.get("x0", None) if setup else args[0]
                        getattr(cb, f"on_{func.__name__}_end")(self, x)
                return ret

            return wrapper

        for method in ["setup", "step", "run"]:
            setattr(self, method, cbdecorator(getattr(self, method), method == "setup"))

    @abstractmethod
    def memory_usage(self, *args, **kwargs):
        pass

    @abstractmethod
    def setup(self, *args, **kwargs):
        pass

    @abstractmethod
    def step(self, *args, **kwargs):
        pass

    @abstractmethod
    def run(self, *args, **kwargs):
        pass

    @abstractmethod
    def finalize(self, *args, **kwargs):
        pass

    @abstractmethod
    def solve(self, *args, **kwargs):
        pass

    def callback(self, x, *args, **kwargs) -> None:
        """User hook called after every step (``basesolver.py:303-330``)."""
        pass
