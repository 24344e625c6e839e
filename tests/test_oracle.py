"""CPU tests: the oracle against the reference's own outputs (tests/golden).

The goldens were produced by running the reference package (tests/golden/make_golden.py).
These tests pin the restatement before it is trusted as the checker of the CUDA path.
"""
import numpy as np
import pytest

from cases import SOLVE_CASES, SWEEP_CASES
from oracle.fp64 import d_eff_fp64
from oracle.percolation import spans_axis0
from oracle.sor import OracleSolve

SMALL_SOLVES = [k for k in SOLVE_CASES if not k.startswith("bernoulli")]


@pytest.mark.parametrize("name", list(SWEEP_CASES))
def test_oracle_half_sweeps_bitwise(name, golden):
    kind, make, kw, n = SWEEP_CASES[name]
    o = OracleSolve(make(), kind=kind, **kw)
    o.half_sweep(n)
    ref = golden[f"{name}/field"]
    # bitwise up to the sign of zero (x == y compares -0.0 equal to 0.0)
    assert np.array_equal(o.field, ref)


@pytest.mark.parametrize("name", SMALL_SOLVES + ["bernoulli100"])
def test_oracle_solve_matches_reference(name, golden):
    kind, make, kw, solve_kw, _ = SOLVE_CASES[name]
    o = OracleSolve(make(), kind=kind, **kw)
    o.solve(**solve_kw)
    assert o.iter == int(golden[f"{name}/iter"])
    assert bool(o.converged) == bool(golden[f"{name}/converged"])
    tau_ref = golden[f"{name}/tau"]
    assert np.array_equal(np.isinf(o.tau), np.isinf(tau_ref))
    fin = np.isfinite(tau_ref)
    # the oracle reduces layer means in float64, the reference in float32
    np.testing.assert_allclose(o.tau[fin], tau_ref[fin], rtol=2e-6)
    if o.electrode:
        np.testing.assert_array_equal(o.k_0, golden[f"{name}/k_0"])
        np.testing.assert_array_equal(o.a_x, golden[f"{name}/a_x"])
        np.testing.assert_allclose(o.c_x, golden[f"{name}/c_x"], rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(o.k_x, golden[f"{name}/k_x"], rtol=1e-3, atol=1e-3)
        return
    d_ref = golden[f"{name}/D_eff"]
    np.testing.assert_allclose(o.D_eff, d_ref, rtol=2e-6, atol=1e-9)
    np.testing.assert_allclose(o.flux_1d, golden[f"{name}/flux_1d"], rtol=1e-4, atol=1e-7)


def test_reference_known_answers_through_oracle(golden):
    """The reference test-suite's own pins (tests/test_taufactor.py) hold for the oracle."""
    o = OracleSolve(SOLVE_CASES["slanted"][1](), kind="binary")
    o.solve()
    assert np.around(o.tau, decimals=5) == 7.51667
    for name in ("blocks_cube", "blocks_long_x", "blocks_long_z", "strip", "p_blocks", "p_strip"):
        kind, make, kw, skw, _ = SOLVE_CASES[name]
        o = OracleSolve(make(), kind=kind, **kw)
        o.solve(**skw)
        assert np.around(o.tau, decimals=5) == 1.0
    for name in ("nonperc", "deadend", "p_nonperc", "mp_nonperc"):
        kind, make, kw, skw, _ = SOLVE_CASES[name]
        o = OracleSolve(make(), kind=kind, **kw)
        o.solve(**skw)
        assert np.all(o.tau == np.inf)
        assert np.around(o.D_eff, 5) == 0


@pytest.mark.parametrize("name", ["slanted", "strip", "mp_strip12", "mp_strip123", "pmp_slanted", "aniso_slanted",
                                  "blocks_long_x"])
def test_fp64_oracle_matches_reference_known_answers(name, golden):
    kind, make, kw, _, _ = SOLVE_CASES[name]
    o = OracleSolve(make(), kind=kind, **kw)
    d, _, resid = d_eff_fp64(o)
    assert np.all(resid < 1e-9)
    np.testing.assert_allclose(d, golden[f"{name}/D_eff"], rtol=2e-6)


def test_fp64_oracle_bernoulli100(golden):
    """The reference at conv_crit 2e-2 sits ~1e-4 from the FP64 solution of its own operator."""
    o = OracleSolve(SOLVE_CASES["bernoulli100"][1](), kind="binary")
    d, _, resid = d_eff_fp64(o)
    assert resid[0] < 1e-9
    ref = golden["bernoulli100/D_eff"][0]
    assert abs(d[0] - ref) / d[0] < 3e-4
    np.testing.assert_allclose(d[0], 0.10480938, rtol=1e-6)


def test_percolation_restatement():
    m = np.zeros((6, 5, 5), dtype=bool)
    assert not spans_axis0(m)
    m[:, 2, 2] = True
    assert spans_axis0(m)
    m[3, 2, 2] = False
    assert not spans_axis0(m)
    m[2:5, 2, 3] = True  # detour around the gap
    assert spans_axis0(m)


@pytest.mark.parametrize("coefficients", ["f32", "f64"])
def test_fp64_adjoint_gradient_euler_and_finite_differences(coefficients):
    """The FP64 adjoint gradient of a per-voxel conductivity field: Euler's identity
    sum(kappa dD/dkappa) = D_eff (D_eff is homogeneous of degree 1 in kappa) and central
    finite differences (h = 1e-3). With float32 faces D_eff moves in steps of one face rounding,
    so the finite differences only hold to ~1e-3; with float64 faces to the h^2 truncation."""
    from oracle.fp64 import adjoint_gradient_fp64

    kap = (0.05 + np.random.default_rng(71).random((1, 10, 9, 12))).astype(np.float32)
    o = OracleSolve(kap, kind="kappa")
    g = adjoint_gradient_fp64(o, rtol=1e-14, coefficients=coefficients)[0]
    d = d_eff_fp64(o, rtol=1e-14, coefficients=coefficients)[0][0]
    euler = abs(float((kap[0].astype(np.float64) * g).sum()) - d) / d
    assert euler < (1e-13 if coefficients == "f64" else 1e-8), euler
    rng = np.random.default_rng(72)
    for _ in range(3):
        i = tuple(int(rng.integers(0, n)) for n in kap.shape[1:])
        kp, km = kap.copy(), kap.copy()
        kp[(0,) + i] += np.float32(1e-3)
        km[(0,) + i] -= np.float32(1e-3)
        dp = d_eff_fp64(OracleSolve(kp, kind="kappa"), rtol=1e-14, coefficients=coefficients)[0][0]
        dm = d_eff_fp64(OracleSolve(km, kind="kappa"), rtol=1e-14, coefficients=coefficients)[0][0]
        fd = (dp - dm) / (float(kp[(0,) + i]) - float(km[(0,) + i]))
        assert abs(fd - g[i]) / abs(fd) < (1e-5 if coefficients == "f64" else 3e-3), (i, fd, g[i])
