"""GPU parity tests: the sm_103a path against the reference's goldens and the oracle.

Bar: half-sweeps are bitwise equal to the reference (up to the sign of zero); solves reach the
same iteration count and tau/D_eff within 2e-6 relative (the only difference being the float64
layer reduction), i.e. far inside the 1e-3 tolerance against the reference Solver.
"""
import numpy as np
import pytest
import torch

from cases import SOLVE_CASES, SWEEP_CASES, random_binary, random_labels
from oracle.sor import OracleSolve

pytestmark = pytest.mark.gpu

import taufactor_gb300 as tg  # noqa: E402

CLASSES = {
    "binary": tg.Solver,
    "periodic": tg.PeriodicSolver,
    "anisotropic": tg.AnisotropicSolver,
    "multiphase": tg.MultiPhaseSolver,
    "periodic_multiphase": tg.PeriodicMultiPhaseSolver,
    "electrode": tg.ElectrodeSolver,
    "periodic_electrode": tg.PeriodicElectrodeSolver,
}


def make_solver(kind, img, kw):
    cls = CLASSES[kind]
    if kind in ("multiphase", "periodic_multiphase"):
        ds = kw.get("diffusivities")
        return cls(img, dict(ds) if ds is not None else None, device="cuda")
    if kind == "anisotropic":
        return cls(img, kw["spacing"], device="cuda")
    return cls(img, device="cuda")


def interior_and_x_ghosts(f):
    """The parts of the padded field the reference defines independently of ghost timing."""
    f = np.asarray(f)
    return f[:, :, 1:-1, 1:-1]


@pytest.mark.parametrize("name", list(SWEEP_CASES))
def test_half_sweeps_bitwise_vs_reference(name, golden):
    kind, make, kw, n = SWEEP_CASES[name]
    s = make_solver(kind, make(), kw)
    if kind in ("electrode", "periodic_electrode"):
        # the reference's k_0 is a float32 torch mean whose last bit depends on the host
        k_ref = golden[f"{name}/k_0"]
        np.testing.assert_allclose(s.k_0, k_ref, rtol=2.0 ** -22, atol=0)
        s.set_k_0(k_ref)
    s._advance(n)
    got = s.field.cpu().numpy()
    ref = golden[f"{name}/field"]
    assert np.array_equal(interior_and_x_ghosts(got), interior_and_x_ghosts(ref))


@pytest.mark.parametrize("kind", ["binary", "periodic", "anisotropic", "multiphase", "periodic_multiphase",
                                  "electrode", "periodic_electrode"])
@pytest.mark.parametrize("shape", [(1, 23, 40, 70), (2, 9, 17, 33), (1, 5, 64, 128), (1, 30, 8, 16),
                                   (1, 100, 24, 40)])
def test_chunked_half_sweeps_bitwise_vs_oracle(kind, shape):
    """Every chunk length 1..9 (several tiled launches, odd/even colour starts) matches. The
    long-x shape runs each tile column as several x-chunks (few columns for 152 SMs)."""
    seed = sum(shape)
    if kind in ("multiphase", "periodic_multiphase", "electrode", "periodic_electrode"):
        img = random_labels(shape, seed)
        kw = {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.1}}
    else:
        img = random_binary(shape, seed)
        kw = {"spacing": (1.0, 1.3, 0.7)} if kind == "anisotropic" else {}
    o = OracleSolve(img, kind=kind, **kw)
    s = make_solver(kind, img, kw)
    for n in (1, 2, 3, 4, 5, 9, 6, 7, 8):
        s._advance(n)
        o.half_sweep(n)
        assert np.array_equal(interior_and_x_ghosts(s.field.cpu().numpy()), interior_and_x_ghosts(o.field)), n


@pytest.mark.parametrize("name", list(SOLVE_CASES))
def test_solve_matches_reference(name, golden):
    kind, make, kw, solve_kw, _ = SOLVE_CASES[name]
    s = make_solver(kind, make(), kw)
    if kind in ("electrode", "periodic_electrode"):
        np.testing.assert_allclose(s.k_0, golden[f"{name}/k_0"], rtol=2.0 ** -22, atol=0)
        s.set_k_0(golden[f"{name}/k_0"])
    ret = s.solve(verbose=False, **solve_kw)
    assert s.iter == int(golden[f"{name}/iter"])
    assert bool(s.converged) == bool(golden[f"{name}/converged"])
    tau_ref = golden[f"{name}/tau"]
    assert np.array_equal(np.isinf(s.tau), np.isinf(tau_ref))
    fin = np.isfinite(tau_ref)
    np.testing.assert_allclose(s.tau[fin], tau_ref[fin], rtol=2e-6)
    assert ret.shape == golden[f"{name}/tau_x"].shape
    if kind in ("electrode", "periodic_electrode"):
        np.testing.assert_allclose(s.c_x, golden[f"{name}/c_x"], rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(s.k_x, golden[f"{name}/k_x"], rtol=1e-3, atol=1e-3)
        return
    np.testing.assert_allclose(s.D_eff, golden[f"{name}/D_eff"], rtol=2e-6, atol=1e-9)
    np.testing.assert_allclose(s.flux_1d, golden[f"{name}/flux_1d"], rtol=1e-4, atol=1e-7)


def test_reference_known_answers():
    """tests/test_taufactor.py pins, through the drop-in classes."""
    img = SOLVE_CASES["slanted"][1]()
    s = tg.Solver(img)
    s.solve(verbose=False)
    assert np.around(s.tau, decimals=5) == 7.51667
    img = np.zeros((10, 50, 50))
    img[:8, 25, 25] = 1
    s = tg.Solver(img)
    s.solve(verbose=False)
    assert np.around(s.D_eff, decimals=5) == 0 and s.tau == np.inf
    s_bin = tg.Solver(img := SOLVE_CASES["slanted"][1](), device="cuda")
    s_bin.solve(iter_limit=1000, verbose=False)
    s_mp = tg.MultiPhaseSolver(img, device="cuda")
    s_mp.solve(iter_limit=1000, verbose=False)
    assert np.isclose(float(s_bin.tau[0]), float(s_mp.tau[0]), atol=1e-3)


def test_batched_matches_single():
    a = random_binary((24, 20, 28), 5)
    b = random_binary((24, 20, 28), 6)
    sb = tg.Solver(np.stack([a, b]))
    sb.solve(verbose=False, conv_crit=1e-3)
    for i, img in enumerate((a, b)):
        s = tg.Solver(img)
        s.solve(verbose=False, conv_crit=1e-3, iter_limit=sb.iter)
        np.testing.assert_allclose(s.D_eff[0], sb.D_eff[i], rtol=1e-3)


def test_solver_matches_oracle_solve_bernoulli100(golden):
    """The 100^3 Bernoulli(0.5) workload: same iterations and D_eff as the reference."""
    img = SOLVE_CASES["bernoulli100"][1]()
    s = tg.Solver(img)
    s.solve(verbose=False, conv_crit=2e-2)
    assert s.iter == 600
    assert abs(s.D_eff[0] - golden["bernoulli100/D_eff"][0]) / golden["bernoulli100/D_eff"][0] < 1e-5


def test_large_volume_properties():
    """256^3 checks that need no CPU solve: exact answers and mirror symmetry."""
    n = 256
    img = np.zeros((n, n, n), dtype=np.uint8)
    img[:, : n // 2, : n // 4] = 1
    s = tg.Solver(img)
    s.solve(verbose=False)
    assert np.around(s.tau, 4) == 1.0
    np.testing.assert_allclose(s.D_eff, 0.125, rtol=1e-5)
    vol = random_binary((1, 64, 256, 256), 9, p=0.7)
    s1 = tg.PeriodicSolver(vol)
    s2 = tg.PeriodicSolver(np.ascontiguousarray(vol[:, :, ::-1, ::-1]))
    # the mirror reverses the order of the y and z neighbour additions, so the two solves agree
    # to rounding, not bitwise
    s1.solve(verbose=False, conv_crit=1e-3)
    s2.solve(verbose=False, conv_crit=1e-3)
    np.testing.assert_allclose(s1.D_eff, s2.D_eff, rtol=2e-4)


def test_field_roundtrip_and_resume():
    img = random_binary((20, 18, 22), 21)
    s = tg.Solver(img)
    s._advance(30)
    f = s.field
    o = OracleSolve(img)
    o.half_sweep(30)
    s2 = tg.Solver(img)
    s2.field = f
    s2.iter = 30
    s2._advance(17)
    o.half_sweep(17)
    assert np.array_equal(s2.field.cpu().numpy()[:, :, 1:-1, 1:-1], o.field[:, :, 1:-1, 1:-1])


def test_bad_arguments_raise():
    from taufactor_gb300._capi import check

    s = tg.Solver(random_binary((8, 8, 8), 1))
    rc = s._lib.tf_advance(None, None, None, None, None, 0, 1, None, None, None)
    with pytest.raises(ValueError):
        check(rc, "tf_advance")


def test_small_integer_division_is_ieee():
    """The binary update divides by nn with one multiply and two FMAs; check every finite input."""
    from taufactor_gb300 import _capi

    lib = _capi.load()
    bad = torch.zeros(9, dtype=torch.int64, device="cuda")
    for n in range(1, 9):
        _capi.check(lib.tf_check_small_division(n, bad[n:].data_ptr(), torch.cuda.current_stream().cuda_stream),
                    "tf_check_small_division")
    assert bad.cpu().tolist() == [0] * 9


@pytest.mark.parametrize("k_max", [2, 3, 4])
@pytest.mark.parametrize("tile", [0, 1, 2])
@pytest.mark.parametrize("kind", ["binary", "periodic"])
@pytest.mark.parametrize("shape", [(2, 21, 52, 136), (1, 150, 20, 40)])
def test_tile_variants_bitwise(kind, tile, k_max, shape):
    """Every tile shape and fused depth of the kernel gives the reference iterations bit for bit;
    the second shape splits every tile column into 4-8 x-chunks of uneven length."""
    img = random_binary(shape, 31 + tile)
    o = OracleSolve(img, kind=kind)
    s = make_solver(kind, img, {})
    s._op.tile = tile
    s._op.k_max = k_max
    for n in (4, 4, 3, 8, 1, 12):
        s._advance(n)
        o.half_sweep(n)
        assert np.array_equal(interior_and_x_ghosts(s.field.cpu().numpy()), interior_and_x_ghosts(o.field)), n


@pytest.mark.parametrize("k_max", [2, 4])
@pytest.mark.parametrize("kind", ["binary", "periodic"])
@pytest.mark.parametrize("shape", [(2, 21, 52, 136), (1, 150, 20, 40), (2, 23, 38, 102), (1, 30, 19, 131),
                                   (1, 9, 260, 256)])
def test_row_pair_tile_bitwise(kind, k_max, shape):
    """Tile shape 3 (row pairs, even fused depths; odd counts run on shape 1) gives the reference
    iterations bit for bit: partial tiles in y and z, odd half-row lengths, periodic faces whose
    half-row length is odd (cell-by-cell ghost copies), both colour starts and x-chunked columns."""
    img = random_binary(shape, 77 + k_max)
    o = OracleSolve(img, kind=kind)
    s = make_solver(kind, img, {})
    s._op.tile = 3
    s._op.k_max = k_max
    for n in (4, 4, 2, 8, 3, 6, 12, 1, 4):
        s._advance(n)
        o.half_sweep(n)
        assert np.array_equal(interior_and_x_ghosts(s.field.cpu().numpy()), interior_and_x_ghosts(o.field)), n


@pytest.mark.parametrize("p", [0.25, 0.31, 0.4])
def test_device_spanning_test_matches_host_labelling(p):
    """tf_spans_x (union-find on the device) agrees with the host's face-connected labelling on
    random masks near the site-percolation threshold, in batches of uneven outcome."""
    from taufactor_gb300.percolation import spans_x

    for seed, shape in enumerate([(6, 21, 17, 19), (3, 40, 9, 33), (2, 9, 64, 48)]):
        img = (np.random.default_rng(1000 * seed + int(100 * p)).random(shape) < p).astype(np.uint8)
        s = tg.Solver(img)
        got = s.spans_x_device()
        want = np.array([spans_x(img[b] == 1) for b in range(shape[0])])
        assert np.array_equal(got, want), (shape, got, want)


def test_device_spanning_test_long_path():
    """A single serpentine path through every row (long union-find chains) and its cut copy."""
    from taufactor_gb300.percolation import spans_x

    img = np.zeros((64, 66, 33), dtype=np.uint8)
    for x in range(64):
        img[x, x, :] = 1  # one row per plane, joined to the next plane's row at alternating ends
        if x + 1 < 64:
            img[x + 1, x, 32 if x % 2 else 0] = 1
    assert spans_x(img == 1)
    cut = img.copy()
    cut[40] = 0
    for v in (img, cut):
        s = tg.Solver(v)
        assert bool(s.spans_x_device()[0]) == spans_x(v == 1)
    mp = tg.MultiPhaseSolver(np.where(img == 1, 2, 0).astype(np.uint8), {0: 0.0, 2: 0.7})
    assert bool(mp.spans_x_device()[0])


def test_device_label_pass_matches_host_set_up():
    """uint8 / bool labels are checked and counted on the device (tf_label_stats): vol_x equals
    the host computation for ragged plane sizes (unaligned plane starts), the solve equals the
    one set up from int64 labels (host path), and labels other than 0/1 raise the reference's
    ValueError."""
    from taufactor_gb300.solvers import plane_fraction

    for shape, seed in (((2, 9, 7, 13), 31), ((1, 20, 33, 17), 32), ((3, 16, 16, 16), 33)):
        img = random_binary(shape, seed)
        a = tg.Solver(img)
        assert np.array_equal(a.vol_x, plane_fraction(img == 1))
        b = tg.Solver(img.astype(np.int64))  # host set-up
        assert np.array_equal(a.vol_x, b.vol_x)
        a.solve(verbose=False, conv_crit=1e-3)
        b.solve(verbose=False, conv_crit=1e-3)
        assert a.iter == b.iter and np.array_equal(a.D_eff, b.D_eff)
        c = tg.Solver(img.astype(bool))
        assert np.array_equal(c.vol_x, a.vol_x)
    bad = random_binary((6, 6, 6), 34)
    bad[3, 3, 3] = 2
    with pytest.raises(ValueError, match="Input image must only contain 0s and 1s"):
        tg.Solver(bad)
