"""The drop-in boundary on the GPU: float64 precision against the reference's own float64 runs,
and the operator tensors (factor, cb, D_x/D_y/D_z) against the oracle's restatement of the
reference's set-up (taufactor/taufactor.py:24-67, :218-225, :402-410, :459-471, :493-499,
:577-604, :626-650)."""
import os
import sys

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from cases import DOUBLE_CASES, random_binary, random_labels  # noqa: E402
from oracle.sor import OracleSolve  # noqa: E402

import taufactor_gb300 as tg  # noqa: E402
from taufactor_gb300.solvers import ThroughTransportSolver  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(HERE, "golden", "fullsize_outputs.npz")


def double_solver(base):
    """The reference's way to sweep in float64: its public classes take no precision argument,
    its base ThroughTransportSolver does (taufactor.py:278-280); this repeats Solver.__init__."""
    class DoubleSolver(base):
        def __init__(self, img, omega=None, D_0=1, device="cuda"):
            self._check_binary_labels(img)
            self.conductive_labels = [1]
            ThroughTransportSolver.__init__(self, img, omega=omega, precision=torch.float64, device=device)
            self.D_0 = D_0
            self.D_mean = np.mean(self.vol_x, axis=1)

    return DoubleSolver


@pytest.mark.parametrize("name", sorted(DOUBLE_CASES))
def test_float64_precision_matches_reference(name):
    """precision=torch.float64: float32 sweeps plus the float64 correction give D_eff within 1e-3
    of the reference's float64 sweeps at its own conv_crit, and a float64 field."""
    g = np.load(GOLDEN)
    kind, make, solve_kw = DOUBLE_CASES[name]
    cls = double_solver(tg.PeriodicSolver if kind == "periodic" else tg.Solver)
    s = cls(make())
    s.solve(verbose=False, **solve_kw)
    assert s.precision == torch.float64 and s.converged
    np.testing.assert_allclose(s.D_eff, g[f"{name}/D_eff"], rtol=1e-3)
    assert s.residual_history[-1] < 1e-10
    f = s.field
    assert f.dtype == torch.float64 and f.shape == (s.batch_size, s.Nx + 2, s.Ny + 2, s.Nz + 2)
    # Dirichlet planes 2 bc over the interior y/z extent (their y/z edges are 0, as _pad leaves them)
    assert torch.all(f[:, 0, 1:-1, 1:-1] == -1.0) and torch.all(f[:, -1, 1:-1, 1:-1] == 1.0)


@pytest.mark.parametrize("kind", ["binary", "periodic", "anisotropic"])
def test_factor_and_cb_match_reference_setup(kind):
    img = random_binary((2, 9, 12, 10), 5)
    spacing = (1.0, 1.3, 0.7)
    if kind == "anisotropic":
        s = tg.AnisotropicSolver(img, spacing)
        o = OracleSolve(img, kind=kind, spacing=spacing)
    else:
        s = (tg.PeriodicSolver if kind == "periodic" else tg.Solver)(img)
        o = OracleSolve(img, kind=kind)
    assert s.factor.dtype == torch.float32
    assert np.array_equal(s.factor.cpu().numpy(), o.factor)
    for i in range(2):
        assert np.array_equal(s.cb[i].cpu().numpy(), o.cb[i])


@pytest.mark.parametrize("kind", ["multiphase", "periodic_multiphase"])
def test_multiphase_faces_match_reference_setup(kind):
    img = random_labels((2, 8, 11, 9), 6)
    ds = {0: 0.0, 1: 1.0, 2: 0.3}
    s = (tg.PeriodicMultiPhaseSolver if kind == "periodic_multiphase" else tg.MultiPhaseSolver)(img, dict(ds))
    o = OracleSolve(img, kind=kind, diffusivities=dict(ds))
    for name in ("D_x", "D_y", "D_z", "factor"):
        assert np.array_equal(getattr(s, name).cpu().numpy(), getattr(o, name)), name
