"""Solver template with the life cycle of ``pylops/optimization/basesolver.py:18-330``.

A solver subclasses :class:`Solver` and implements ``setup``, ``step``,
``run``, ``finalize``, ``solve`` and ``memory_usage``.  Callbacks observe
``setup``, ``step`` and ``run``: every callback's ``on_<name>_begin`` runs
before the method, in list order, and every ``on_<name>_end`` after it, in
reverse list order (basesolver.py:80-120).  The model handed to a callback
is the ``x0`` keyword for ``setup`` and the first positional argument for
``step`` and ``run``.

Here the hooks are installed once per class, when a subclass is defined
(``__init_subclass__``), instead of re-wrapping bound methods on every
instance.  A method that calls the same method of its parent class
(``super().step(x)``) notifies the callbacks once, as an instance-level
wrapper of the outermost method would: a per-instance depth counter lets
only the outermost call of a given name notify.
"""

import time
from abc import ABCMeta, abstractmethod

__all__ = ["Solver"]

_units = {"B": 1, "KB": 1024, "MB": 1024 ** 2, "GB": 1024 ** 3}

_OBSERVED = ("setup", "step", "run")


def _observed(name, method):
    """``method`` with the callbacks' begin/end hooks of ``name`` around it."""

    def hooked(self, *args, **kwargs):
        depth = self.__dict__.setdefault("_hook_depth", {})
        outer = depth.get(name, 0) == 0
        hooks = self.callbacks if (outer and self.callbacks) else ()
        model = kwargs.get("x0") if name == "setup" else (args[0] if args else None)
        for cb in hooks:
            getattr(cb, "on_" + name + "_begin")(self, model)
        depth[name] = depth.get(name, 0) + 1
        try:
            out = method(self, *args, **kwargs)
        finally:
            depth[name] -= 1
        for cb in reversed(list(hooks)):
            getattr(cb, "on_" + name + "_end")(self, model)
        return out

    hooked.__name__ = method.__name__
    hooked.__qualname__ = method.__qualname__
    hooked.__doc__ = method.__doc__
    hooked.__wrapped__ = method
    return hooked


class Solver(metaclass=ABCMeta):
    """Base class: the setup/step/run/finalize/solve life cycle, the shared
    banner printing and the callback hooks of the reference's template."""

    def __init_subclass__(cls, **kwargs):
        super().__init_subclass__(**kwargs)
        for name in _OBSERVED:
            fn = cls.__dict__.get(name)
            if fn is not None and not getattr(fn, "__isabstractmethod__", False):
                setattr(cls, name, _observed(name, fn))

    def __init__(self, Op, callbacks=None) -> None:
        self.Op = Op
        self.callbacks = callbacks
        self.iiter = 0
        self.tstart = time.time()

    # banner text shared by the solvers (the wording is part of their output)
    def _print_solver(self, text: str = "", nbar: int = 80) -> None:
        rows, cols = self.Op.shape
        print(type(self).__name__ + text)
        print("-" * nbar)
        print(f"The Operator Op has {rows} rows and {cols} cols")

    def _print_setup(self, *args, **kwargs) -> None:
        pass

    def _print_step(self, *args, **kwargs) -> None:
        pass

    def _print_finalize(self, *args, nbar: int = 80, **kwargs) -> None:
        print()
        print(f"Iterations = {self.iiter}        Total time (s) = {self.telapsed:.2f}")
        print("-" * nbar)
        print()

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
