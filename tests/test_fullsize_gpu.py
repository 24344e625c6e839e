"""Benchmark-size parity: volumes of the benchmark workloads solved through the drop-in classes
at the benchmark's kernel configuration (16 x 128 tiles, 4 half-sweeps per launch), against the
reference's own solve of the same volume and against the FP64 solution of the same operator.

The fixtures (tests/golden/fullsize_outputs.npz, made by ``make_golden.py fullsize``) hold the
reference's iteration count, D_eff, tau and layer flux (taufactor/taufactor.py:156-191,
:293-331) and the FP64 D_eff from oracle/fp64.py (CG to a relative residual of 1e-10). The
volumes are regenerated here from their seeds.

Bars: the same iteration count as the reference (its convergence rule, checked every 100
half-sweeps); D_eff within 2e-6 of the reference's (float64 against float32 layer means); the
layer flux within 1e-5 of its largest value; after FP64 defect correction, D_eff within 1e-8 of
the FP64 solution.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from cases import FULLSIZE_CASES  # noqa: E402

import taufactor_gb300 as tg  # noqa: E402
from taufactor_gb300.autotune import apply  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(HERE, "golden", "fullsize_outputs.npz")


def _solver(kind, img, kw):
    if kind == "multiphase":
        return tg.MultiPhaseSolver(img, dict(kw["diffusivities"]))
    return (tg.PeriodicSolver if kind == "periodic" else tg.Solver)(img)


@pytest.mark.parametrize("name", sorted(FULLSIZE_CASES))
def test_benchmark_size_volume_matches_reference_and_fp64(name):
    g = np.load(GOLDEN)
    kind, make, kw, solve_kw, _ = FULLSIZE_CASES[name]
    img = make()
    tiles = [1, 3] if kind == "binary" else [0]  # the binary benchmark tiles; shape 0 for the others
    for tile in tiles:
        s = _solver(kind, img, kw)
        apply(s, tile, 4)
        s.solve(verbose=False, **solve_kw)
        assert s.converged == bool(g[f"{name}/converged"])
        assert s.iter == int(g[f"{name}/iter"]), (tile, s.iter)
        np.testing.assert_allclose(s.D_eff, g[f"{name}/D_eff"], rtol=2e-6)
        np.testing.assert_allclose(s.tau, g[f"{name}/tau"], rtol=2e-6)
        ref_flux = g[f"{name}/flux_1d"]
        assert np.max(np.abs(s.flux_1d - ref_flux)) <= 1e-5 * np.max(np.abs(ref_flux))
        hist = s.refine(tol=1e-12, max_outer=40)
        assert hist[-1] < 1e-12
        np.testing.assert_allclose(s.D_eff, g[f"{name}/D_eff_fp64"], rtol=1e-8)
