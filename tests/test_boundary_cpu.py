"""The drop-in boundary without a GPU: the `precision` argument and the reference's hook
protocol (taufactor/taufactor.py:24-103)."""
import numpy as np
import pytest
import torch

import taufactor_gb300 as tg
from taufactor_gb300.solvers import SORSolver, ThroughTransportSolver


def test_precision_values():
    img = np.ones((4, 4, 4), dtype=np.uint8)
    # only float32 and float64 are meaningful; anything else is refused before the device is touched
    for bad in (torch.float16, torch.int32, "double"):
        with pytest.raises(ValueError, match="precision"):
            ThroughTransportSolver(img, precision=bad, device="cuda")
    # the public classes take no precision argument, as in the reference (taufactor.py:380)
    with pytest.raises(TypeError):
        tg.Solver(img, precision=torch.float64)


@pytest.mark.parametrize("hook", SORSolver.DEVICE_HOOKS)
def test_overridden_hooks_are_refused(hook):
    """A subclass overriding a hook of the reference's SORSolver would be ignored by the CUDA
    kernels: construction fails with NotImplementedError naming the hook."""
    cls = type("Custom", (tg.Solver,), {hook: lambda self, *a: None})
    with pytest.raises(NotImplementedError, match=hook):
        cls(np.ones((4, 4, 4), dtype=np.uint8), device="cuda")


def test_overriding_other_methods_is_allowed_up_to_the_device():
    """compute_metrics and other host-side methods may be overridden; construction then proceeds
    to the device check (RuntimeError here: no CUDA device in this container)."""
    class Custom(tg.Solver):
        def compute_metrics(self):
            return super().compute_metrics()

    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    with pytest.raises(RuntimeError):
        Custom(np.ones((4, 4, 4), dtype=np.uint8), device="cuda")
