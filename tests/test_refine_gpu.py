"""GPU tests of the FP64 defect correction against the FP64 oracle (scipy CG to 1e-10).

Tolerance: refined D_eff within 1e-8 relative of the oracle (both solve the same operator to a
relative residual <= 1e-10); the accuracy bar of a converged solve is 1e-4.
"""
import numpy as np
import pytest

from cases import SOLVE_CASES, random_binary, random_labels
from oracle.fp64 import d_eff_fp64
from oracle.sor import OracleSolve

pytestmark = pytest.mark.gpu

import taufactor_gb300 as tg  # noqa: E402


def _solver(kind, img, kw):
    if kind == "binary":
        return tg.Solver(img)
    if kind == "periodic":
        return tg.PeriodicSolver(img)
    if kind == "anisotropic":
        return tg.AnisotropicSolver(img, kw["spacing"])
    if kind == "multiphase":
        return tg.MultiPhaseSolver(img, dict(kw["diffusivities"]))
    return tg.PeriodicMultiPhaseSolver(img, dict(kw["diffusivities"]))


CASES = [
    ("binary", lambda: SOLVE_CASES["slanted"][1](), {}),
    ("binary", lambda: random_binary((2, 24, 20, 28), 41, 0.65), {}),
    ("periodic", lambda: random_binary((24, 20, 28), 42, 0.6), {}),
    # (odd periodic sizes are left out: there red-black couples equal colours across the wrap and
    # the reference iteration itself diverges at its default omega; see test_rhs_half_sweeps_bitwise
    # for the odd-size path)
    ("periodic", lambda: random_binary((21, 18, 22), 43, 0.6), {}),
    ("anisotropic", lambda: random_binary((22, 18, 26), 44, 0.65), {"spacing": (1.0, 1.3, 0.7)}),
    ("multiphase", lambda: random_labels((22, 20, 24), 45), {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.1}}),
    ("periodic_multiphase", lambda: random_labels((20, 18, 22), 46),
     {"diffusivities": {0: 0.05, 1: 1.0, 2: 0.3}}),
]


@pytest.mark.parametrize("kind,make,kw", CASES)
def test_refined_d_eff_matches_fp64_oracle(kind, make, kw):
    img = make()
    s = _solver(kind, img, kw)
    s.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-11})
    assert s.residual_history[-1] < 1e-11, s.residual_history
    o = OracleSolve(img, kind=kind, **kw)
    d64, _, resid = d_eff_fp64(o, rtol=1e-11)
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-8, atol=1e-14)


def test_refinement_reduces_residual_monotonically():
    s = tg.Solver(random_binary((40, 36, 44), 47, 0.6))
    s.solve(verbose=False, conv_crit=1e-2)
    hist = s.refine(tol=1e-12)
    assert hist[-1] < 1e-12
    assert all(b < a for a, b in zip(hist, hist[1:]))


@pytest.mark.parametrize("kind,shape,kw", [
    ("binary", (2, 13, 18, 40), {}),
    ("periodic", (12, 16, 40), {}),
    ("periodic", (11, 9, 13), {}),
    ("anisotropic", (12, 14, 34), {"spacing": (1.0, 1.3, 0.7)}),
    ("multiphase", (12, 14, 34), {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.1}}),
])
def test_rhs_half_sweeps_bitwise(kind, shape, kw):
    """Correction sweeps (A e = r, homogeneous faces) equal the oracle's iteration with rhs."""
    import ctypes as C

    import torch
    from taufactor_gb300._capi import TfOperator, check

    img = random_labels(shape, 51) if "multiphase" in kind else random_binary(shape, 51, 0.6)
    s = _solver(kind, img, kw)
    o = OracleSolve(img, kind=kind, **kw)
    rng = np.random.default_rng(52)
    rhs = rng.standard_normal(o.field[:, 1:-1, 1:-1, 1:-1].shape).astype(np.float32) * 0.1
    # homogeneous Dirichlet faces and a zero start on both sides
    o.field[:] = 0
    o.top_bc = o.bot_bc = 0.0
    s.field = torch.zeros_like(s.field)
    op0 = TfOperator.from_buffer_copy(s._op)
    op0.ghost_lo = op0.ghost_hi = 0.0
    padded = np.zeros(o.field.shape, dtype=np.float32)
    padded[:, 1:-1, 1:-1, 1:-1] = rhs
    r_split = torch.zeros_like(s._cur)
    check(s._lib.tf_repack(C.byref(s._geom), C.byref(op0), torch.from_numpy(padded).cuda().data_ptr(),
                           r_split.data_ptr(), s._stream()), "tf_repack")
    for n in (4, 5, 3):
        in_b = C.c_int(0)
        check(s._lib.tf_advance_rhs(C.byref(s._geom), C.byref(op0), s._cur.data_ptr(), s._other.data_ptr(),
                                    s._code.data_ptr(), r_split.data_ptr(), o.iter % 2, n, s._err.data_ptr(),
                                    C.byref(in_b), s._stream()), "tf_advance_rhs")
        if in_b.value:
            s._cur, s._other = s._other, s._cur
        o.half_sweep(n, rhs=rhs)
        out = torch.empty(o.field.shape, dtype=torch.float32, device="cuda")
        check(s._lib.tf_unpack(C.byref(s._geom), C.byref(op0), s._cur.data_ptr(), out.data_ptr(), s._stream()),
              "tf_unpack")
        got = out.cpu().numpy()[:, :, 1:-1, 1:-1]
        assert np.array_equal(got, o.field[:, :, 1:-1, 1:-1]), n


def _pocket_volume():
    """Three labels (blurred, seed 48) with a conductive pocket sealed inside a shell of the
    zero-conductivity label: a cluster that touches neither x-face."""
    from cases import _blur_labels

    img = _blur_labels((30, 24, 28), 48)
    img[10:20, 8:16, 8:16] = 0
    img[12:18, 10:14, 10:14] = 1
    return img


def _wrap_path_volume():
    """Label 1 channels in label 0 (conductivity 0): the only path from x = 0 to x = nx - 1 runs
    through a middle segment that touches the others across the periodic y face alone."""
    img = np.zeros((24, 12, 10), dtype=np.uint8)
    img[:9, 0:2, 3:6] = 1      # touches x = 0
    img[7:17, 10:12, 3:6] = 1  # middle segment: rows 10-11 wrap onto rows 0-1
    img[15:, 0:2, 3:6] = 1     # touches x = nx - 1
    return img


@pytest.mark.parametrize("kind,make,ds", [
    ("multiphase", _pocket_volume, {0: 0.0, 1: 1.0, 2: 0.1}),
    ("periodic_multiphase", _pocket_volume, {0: 0.0, 1: 1.0, 2: 0.1}),
    ("periodic_multiphase", _wrap_path_volume, {0: 0.0, 1: 1.0}),
    ("anisotropic", lambda: (_pocket_volume() > 0).astype(np.uint8), None),
])
def test_refinement_with_unanchored_clusters_reaches_tight_tolerance(kind, make, ds):
    """With float32 faces the diagonal is a rounded sum, so the block of a cluster touching
    neither x-face is nearly singular; the refinement solves the anchored system (as the FP64
    oracle does) and reaches 1e-12, and clusters joined across a periodic face stay in it."""
    img = make()
    kw = {"spacing": (1.0, 1.3, 0.7)} if kind == "anisotropic" else {"diffusivities": ds}
    s = _solver(kind, img, kw)
    s.solve(verbose=False, conv_crit=1e-3)
    hist = s.refine(tol=1e-12, max_outer=20)
    assert hist[-1] < 1e-12, hist
    o = OracleSolve(img, kind=kind, **kw)
    d64, _, _ = d_eff_fp64(o, rtol=1e-12)
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-9, atol=1e-14)


def test_refinement_with_its_own_omega_reaches_the_same_solution():
    """The correction sweeps may over-relax with their own omega (no reference counterpart): the
    refined system and its D_eff do not change, only the rate."""
    img = random_binary((40, 32, 36), 53, 0.6)
    a = tg.Solver(img)
    a.solve(verbose=False, conv_crit=1e-3)
    ha = a.refine(tol=1e-12, max_outer=30)
    b = tg.Solver(img)
    b.solve(verbose=False, conv_crit=1e-3)
    hb = b.refine(tol=1e-12, max_outer=30, omega=2 - 3 / img.shape[0])
    assert ha[-1] < 1e-12 and hb[-1] < 1e-12
    np.testing.assert_allclose(b.D_eff, a.D_eff, rtol=1e-11, atol=0)


@pytest.mark.parametrize("kind", ["electrode", "periodic_electrode"])
def test_electrode_refinement_matches_fp64_oracle(kind):
    """ElectrodeSolver's FP64 defect correction (divisor nn + nr k_0, inlet Dirichlet term,
    closed outlet) reaches a relative residual of 1e-12, and its tau and k_x equal those of the
    FP64 oracle's solution of the same operator (oracle/fp64.py electrode_fp64, float64 layer
    means) to 1e-8."""
    from oracle.fp64 import electrode_fp64

    img = (np.random.default_rng(5).random((2, 20, 12, 14)) < 0.6).astype(np.uint8)
    cls = tg.PeriodicElectrodeSolver if kind == "periodic_electrode" else tg.ElectrodeSolver
    s = cls(img)
    o = OracleSolve(img, kind=kind)
    s.set_k_0(o.k_0)  # the same float32 reaction prefactors on both sides
    s.solve(verbose=False, conv_crit=1e-3)
    hist = s.refine(tol=1e-12, max_outer=60)
    assert hist[-1] < 1e-12
    o.field = s.field.cpu().numpy()  # the float32 solution; the oracle replaces its anchored part
    tau64, kx64 = electrode_fp64(o)
    np.testing.assert_allclose(s.tau, tau64, rtol=1e-8)
    np.testing.assert_allclose(s.k_x, kx64, rtol=1e-7, atol=1e-10)
