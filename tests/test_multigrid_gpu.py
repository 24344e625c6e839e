"""GPU tests of the multigrid-preconditioned conjugate-gradient inner solve (KappaSolver).

Bars: the coarse faces and factor equal a numpy restatement of the aggregation rule (sums of
fine faces across each coarse interface, halved along a halved normal axis) on even, odd,
periodic and semi-coarsened shapes; the V-cycle is a symmetric preconditioner (<u, M v> =
<M u, v> to float32 rounding); PCG reaches its relative residual with the true residual A x - r
to match; D_eff refined with multigrid inner solves is within 1e-9 of the FP64 oracle, as with
SOR inner solves, also from the initial profile without the float32 loop (solve(method="mg"));
the adjoint gradient with multigrid inner solves is within 1e-6 of the FP64 oracle's.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle.fp64 import adjoint_gradient_fp64, d_eff_fp64
from oracle.sor import OracleSolve

pytestmark = pytest.mark.gpu

import taufactor_gb300 as tg  # noqa: E402
from taufactor_gb300._capi import check  # noqa: E402

HY, HJ = 4, 4


def _kappa(shape, seed, lo=0.05):
    return (lo + np.random.default_rng(seed).random(shape)).astype(np.float32)


def _blurred_kappa(shape, seed, sigma=2.0):
    from scipy.ndimage import gaussian_filter

    logits = gaussian_filter(np.random.default_rng(seed).standard_normal(shape), sigma)
    return (1.0 / (1.0 + np.exp(-2.0 * logits))).astype(np.float32)


class _Layout:
    """Offsets of the split field layout of one tf_geom (the layout every level uses)."""

    def __init__(self, g):
        self.B, self.NX, self.NY, self.NZ, self.ZH = g.batch, g.nx, g.ny, g.nz, g.zh
        self.row = 2 * g.zh
        self.plane = self.row * g.yp
        self.vol = self.plane * g.nx

    def cell(self, b, x, y, z):
        return b * self.vol + x * self.plane + (y + HY) * self.row + (z & 1) * self.ZH + HJ + (z >> 1)

    def xface(self, b, xp, y, z):
        return (b * (self.NX + 1) + xp) * self.plane + (y + HY) * self.row + (z & 1) * self.ZH + HJ + (z >> 1)


def _expected_coarse(fine, cg, fx, fy, fz, periodic, scale=0.5):
    """numpy restatement of tf_mg_coarsen on the coarse interior cells."""
    f, c = _Layout(fine), _Layout(cg)
    sh = [int(c.NX != f.NX), int(c.NY != f.NY), int(c.NZ != f.NZ)]
    k = [np.float32(scale) if s else np.float32(1.0) for s in sh]
    out = {}
    for b in range(c.B):
        for xc in range(c.NX):
            for yc in range(c.NY):
                for zc in range(c.NZ):
                    x0, y0, z0 = xc << sh[0], yc << sh[1], zc << sh[2]
                    xl = x0 + 1 if sh[0] and x0 + 1 < f.NX else x0
                    yl = y0 + 1 if sh[1] and y0 + 1 < f.NY else y0
                    zl = z0 + 1 if sh[2] and z0 + 1 < f.NZ else z0
                    s = [np.float32(0)] * 6
                    for y in range(y0, yl + 1):
                        for z in range(z0, zl + 1):
                            s[0] = np.float32(s[0] + fx[f.xface(b, x0, y, z)])
                            s[1] = np.float32(s[1] + fx[f.xface(b, xl + 1, y, z)])
                    for x in range(x0, xl + 1):
                        for z in range(z0, zl + 1):
                            s[2] = np.float32(s[2] + fy[f.cell(b, x, y0 - 1, z)])
                            s[3] = np.float32(s[3] + fy[f.cell(b, x, yl, z)])
                    for x in range(x0, xl + 1):
                        for y in range(y0, yl + 1):
                            s[4] = np.float32(s[4] + fz[f.cell(b, x, y, z0 - 1)])
                            s[5] = np.float32(s[5] + fz[f.cell(b, x, y, zl)])
                    xm, xp = k[0] * s[0], k[0] * s[1]
                    ym, yp = k[1] * s[2], k[1] * s[3]
                    zm, zp = k[2] * s[4], k[2] * s[5]
                    d = np.float32(xm + xp)
                    for v in (ym, yp, zm, zp):
                        d = np.float32(d + v)
                    if xc == 0:
                        d = np.float32(d + xm)
                    if xc == c.NX - 1:
                        d = np.float32(d + xp)
                    out[(b, xc, yc, zc)] = (xm, xp, yp, zp, d)
    return out


@pytest.mark.parametrize("shape,periodic", [((2, 9, 7, 5), False), ((1, 8, 6, 10), True), ((2, 12, 3, 7), False),
                                            ((1, 6, 8, 4), True)])
def test_coarse_faces_match_numpy(shape, periodic):
    s = tg.KappaSolver(_kappa(shape, 101), periodic=periodic)
    mg = s.multigrid()
    torch.cuda.synchronize()
    for lf, lc in zip(mg.levels[:2], mg.levels[1:3]):
        fx, fy, fz = (t.cpu().numpy() for t in (lf.fx, lf.fy, lf.fz))
        want = _expected_coarse(lf.geom, lc.geom, fx, fy, fz, periodic)
        c = _Layout(lc.geom)
        cfx, cfy, cfz, cdv = (t.cpu().numpy() for t in (lc.fx, lc.fy, lc.fz, lc.dv))
        for (b, x, y, z), (xm, xp, yp, zp, d) in want.items():
            o = c.cell(b, x, y, z)
            got = (cfx[c.xface(b, x, y, z)], cfx[c.xface(b, x + 1, y, z)], cfy[o], cfz[o], cdv[o])
            assert np.array_equal(np.array(got, np.float32), np.array((xm, xp, yp, zp, d), np.float32)), (b, x, y, z)
        # closed ghost rows carry no face and no finite factor
        if not periodic:
            for b in range(c.B):
                assert cfy[c.cell(b, 0, -1, 0)] == 0.0
                assert np.isinf(cdv[c.cell(b, 0, -1, 0)])


def _interior_mask(s):
    m = torch.zeros(s._geom.field_elems, dtype=torch.bool, device="cuda")
    lay = _Layout(s._geom)
    b, x, y, z = np.meshgrid(np.arange(s.batch_size), np.arange(s.Nx), np.arange(s.Ny), np.arange(s.Nz), indexing="ij")
    m[torch.from_numpy(lay.cell(b, x, y, z).ravel()).cuda()] = True
    return m


def _refresh(s, v):
    """periodic ghost copies of a field-layout vector (unpack/repack through the padded form)."""
    pad = torch.empty((s.batch_size, s.Nx + 2, s.Ny + 2, s.Nz + 2), dtype=torch.float32, device="cuda")
    op = s._op
    check(s._lib.tf_unpack(C.byref(s._geom), C.byref(op), v.data_ptr(), pad.data_ptr(), s._stream()), "tf_unpack")
    check(s._lib.tf_repack(C.byref(s._geom), C.byref(op), pad.data_ptr(), v.data_ptr(), s._stream()), "tf_repack")


@pytest.mark.parametrize("periodic", [False, True])
def test_vcycle_is_symmetric(periodic):
    s = tg.KappaSolver(_blurred_kappa((20, 16, 24), 102), periodic=periodic)
    mg = s.multigrid()
    m = _interior_mask(s)
    g = torch.Generator(device="cuda").manual_seed(5)
    u = torch.randn(s._geom.field_elems, device="cuda", generator=g) * m
    v = torch.randn(s._geom.field_elems, device="cuda", generator=g) * m
    mu = mg.vcycle(0, u.clone()).clone()
    mv = mg.vcycle(0, v.clone()).clone()
    a = float((u.double() * mv.double() * m).sum())
    b = float((mu.double() * v.double() * m).sum())
    assert abs(a - b) <= 2e-5 * max(abs(a), abs(b)), (a, b)
    # positive definite on these vectors
    assert float((u.double() * mu.double() * m).sum()) > 0


@pytest.mark.parametrize("periodic", [False, True])
def test_pcg_reaches_true_residual(periodic):
    s = tg.KappaSolver(_blurred_kappa((48, 40, 44), 103), periodic=periodic)
    mg = s.multigrid()
    m = _interior_mask(s)
    r = (torch.randn(s._geom.field_elems, device="cuda", generator=torch.Generator(device="cuda").manual_seed(9))
         * m)
    r0 = r.clone()
    x = torch.zeros_like(r)
    it, rel = mg.solve(x, r, rtol=1e-6, max_iter=100)
    assert rel.max() < 1e-6 and it <= 40, (it, rel)
    if periodic:
        _refresh(s, x)
    ax = torch.zeros_like(x)
    L = mg.levels[0]
    check(s._lib.tf_mg_apply(C.byref(L.geom), x.data_ptr(), L.fx.data_ptr(), L.fy.data_ptr(), L.fz.data_ptr(),
                             L.dv.data_ptr(), ax.data_ptr(), s._stream()), "tf_mg_apply")
    true_rel = float(((ax - r0) * m).double().norm() / (r0 * m).double().norm())
    assert true_rel < 1e-5, true_rel


@pytest.mark.parametrize("kind", ["kappa", "periodic_kappa"])
def test_multigrid_refinement_matches_fp64_oracle(kind):
    kap = _kappa((1, 14, 12, 16), 62)
    o = OracleSolve(kap, kind=kind)
    d64, _, _ = d_eff_fp64(o, rtol=1e-12, coefficients="f64")
    s = tg.KappaSolver(kap, periodic=kind == "periodic_kappa")
    s.solve(conv_crit=1e-3, refine={"tol": 1e-12, "inner": "mg"})
    assert s.residual_history[-1] < 1e-12
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-9)
    g = s.gradient(tol=1e-12, inner="mg").cpu().numpy()
    assert s.adjoint_history[-1] < 1e-12
    gref = adjoint_gradient_fp64(o, rtol=1e-12, coefficients="f64")
    np.testing.assert_allclose(g, gref, rtol=1e-6, atol=1e-8 * np.abs(gref).max())
    # no float32 loop: FP64 correction with multigrid inner solves from the initial profile
    t = tg.KappaSolver(kap, periodic=kind == "periodic_kappa")
    t.solve(method="mg", refine={"tol": 1e-12})
    assert t.converged and t.iter == 0
    np.testing.assert_allclose(t.D_eff, d64, rtol=1e-9)


def test_multigrid_and_sor_inner_solves_agree_on_a_larger_field():
    kap = _blurred_kappa((2, 64, 48, 56), 104)
    a = tg.KappaSolver(kap)
    a.solve(conv_crit=1e-3, refine={"tol": 1e-11, "inner": "sor"})
    ga = a.gradient(tol=1e-11, inner="sor")
    b = tg.KappaSolver(kap)
    b.solve(method="mg", refine={"tol": 1e-11})
    gb = b.gradient(tol=1e-11, inner="mg")
    np.testing.assert_allclose(b.D_eff, a.D_eff, rtol=1e-9)
    torch.testing.assert_close(gb, ga, rtol=1e-6, atol=1e-9 * float(ga.abs().max()))
    assert b.adjoint_history[-1] < 1e-11 and b.residual_history[-1] < 1e-11
    # Euler's identity per volume
    for v in range(2):
        d = float(b.D_eff[v])
        assert abs(float((b.kappa[v].double() * gb[v]).sum()) - d) / d < 1e-9


SOLVER_CASES = [
    ("binary", (2, 24, 20, 28), 41, {}),
    ("periodic", (24, 20, 28), 42, {}),
    ("multiphase", (22, 20, 24), 45, {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.1}}),
    ("periodic_multiphase", (20, 18, 22), 46, {"diffusivities": {0: 0.05, 1: 1.0, 2: 0.3}}),
]


@pytest.mark.parametrize("kind,shape,seed,kw", SOLVER_CASES)
def test_solver_multigrid_refinement_matches_fp64_oracle(kind, shape, seed, kw):
    """refine(inner="mg") of the drop-in solvers (binary and multiphase operators, clusters that
    touch neither x face frozen) reaches the FP64 oracle's D_eff, as refine(inner="sor") does."""
    from cases import random_binary, random_labels

    img = random_binary(shape, seed, 0.6) if kind in ("binary", "periodic") else random_labels(shape, seed)
    make = {"binary": lambda: tg.Solver(img), "periodic": lambda: tg.PeriodicSolver(img),
            "multiphase": lambda: tg.MultiPhaseSolver(img, dict(kw["diffusivities"])),
            "periodic_multiphase": lambda: tg.PeriodicMultiPhaseSolver(img, dict(kw["diffusivities"]))}[kind]
    s = make()
    s.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-11, "inner": "mg"})
    assert s.residual_history[-1] < 1e-11, s.residual_history
    assert len(s.residual_history) <= 5, s.residual_history
    o = OracleSolve(img, kind=kind, **kw)
    d64, _, _ = d_eff_fp64(o, rtol=1e-11)
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-8, atol=1e-14)


def test_solver_multigrid_refinement_of_a_blurred_batch():
    """16-volume-style blurred porous batch (two 96^3 volumes): the multigrid correction reaches
    1e-10 in a few outer steps and agrees with the SOR correction."""
    from taufactor_gb300.synthetic import batch_256

    vols = batch_256(2, 96)
    a = tg.Solver(vols)
    a.solve(verbose=False, conv_crit=1e-2)
    ha = a.refine(tol=1e-10, inner="sor")
    b = tg.Solver(vols)
    b.solve(verbose=False, conv_crit=1e-2)
    hb = b.refine(tol=1e-10, inner="mg")
    assert ha[-1] < 1e-10 and hb[-1] < 1e-10 and len(hb) <= 5, (ha, hb)
    np.testing.assert_allclose(b.D_eff, a.D_eff, rtol=1e-8)


@pytest.mark.parametrize("periodic", [False, True])
def test_kappa_with_zeros_anchored_system_matches_fp64_oracle(periodic):
    """kappa with zeros (clusters cut off from both x faces present): the FP64 steps solve the
    anchored system of the oracle with multigrid inner solves; D_eff within 1e-9 and the
    adjoint gradient within 1e-6 of the oracle's, 0 on the cut-off clusters."""
    rng = np.random.default_rng(105)
    shape = (1, 16, 14, 18)
    kap = ((0.1 + rng.random(shape)) * (rng.random(shape) > 0.4)).astype(np.float32)
    kind = "periodic_kappa" if periodic else "kappa"
    s = tg.KappaSolver(kap, periodic=periodic)
    assert not s.all_positive
    s.solve(conv_crit=1e-3, refine={"tol": 1e-12})
    assert s.residual_history[-1] < 1e-12, s.residual_history
    o = OracleSolve(kap, kind=kind)
    d64, field, _ = d_eff_fp64(o, rtol=1e-12, coefficients="f64")
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-9)
    g = s.gradient(tol=1e-12).cpu().numpy()
    assert s.adjoint_history[-1] < 1e-12
    gref = adjoint_gradient_fp64(o, rtol=1e-12, coefficients="f64")
    np.testing.assert_allclose(g, gref, rtol=1e-6, atol=1e-8 * np.abs(gref).max())
    # the field has conductive voxels outside the anchored system (the oracle leaves them at 0)
    assert np.any((kap > 0) & (field == 0))


def test_multigrid_without_progress_falls_back_to_sor(monkeypatch):
    """A multigrid inner solve that makes no progress (planted on the host) is dropped and the
    SOR sweeps finish the FP64 correction, for KappaSolver and for the drop-in solvers."""
    from cases import random_binary

    from taufactor_gb300.multigrid import KappaMultigrid

    def no_progress(self, x, r, rtol=1e-5, max_iter=200):
        x.zero_()
        return 0, np.ones(self.batch)

    monkeypatch.setattr(KappaMultigrid, "solve", no_progress)
    s = tg.KappaSolver(_kappa((1, 14, 12, 16), 62))
    s.solve(conv_crit=1e-3, refine={"tol": 1e-11})
    assert s.inner_fallback and s.residual_history[-1] < 1e-11
    img = random_binary((2, 24, 20, 28), 41, 0.65)
    t = tg.Solver(img)
    t.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-11, "max_outer": 20})
    assert t.inner_fallback and t.residual_history[-1] < 1e-11
    d64, _, _ = d_eff_fp64(OracleSolve(img, kind="binary"), rtol=1e-11)
    np.testing.assert_allclose(t.D_eff, d64, rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("shape,periodic", [((2, 40, 3, 70), False), ((1, 3, 3, 3), False), ((1, 6, 40, 4), True),
                                            ((3, 33, 17, 9), False)])
def test_multigrid_on_thin_tiny_and_batched_shapes(shape, periodic):
    """Semi-coarsening (extents below 4 kept), a volume with a single level, a periodic slab and
    a batch of three: the multigrid-corrected D_eff matches the FP64 oracle to 1e-9."""
    kap = _blurred_kappa(shape, 106, sigma=1.0)
    s = tg.KappaSolver(kap, periodic=periodic)
    s.solve(method="mg", refine={"tol": 1e-12})
    assert s.converged, s.residual_history
    levels = s.multigrid().levels
    assert all(min(L.dims) >= 1 for L in levels)
    if periodic:  # periodic extents stay even below the finest level
        assert all(L.dims[1] % 2 == 0 and L.dims[2] % 2 == 0 for L in levels[1:])
    else:
        assert max(levels[-1].dims) < 4
    d64, _, _ = d_eff_fp64(OracleSolve(kap, kind="periodic_kappa" if periodic else "kappa"), rtol=1e-12,
                           coefficients="f64")
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-9)


def test_multigrid_refinement_with_a_non_percolating_volume():
    """A batch whose second volume has no path from x = 0 to x = nx - 1 (a solid slab across x;
    the reference's exact-zero test does not catch it, its layer fluxes keep their signs): the
    multigrid correction still reaches the tolerance, the first volume's D_eff matches the FP64
    oracle and the blocked volume's float64 D_eff is zero to rounding."""
    from cases import random_binary

    live = random_binary((20, 16, 24), 107, 0.7)
    dead = random_binary((20, 16, 24), 108, 0.7)
    dead[9:11] = 0  # a solid slab across x
    img = np.stack([live, dead])
    s = tg.Solver(img)
    s.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-11, "inner": "mg"})
    assert s.residual_history[-1] < 1e-11 and not s.inner_fallback
    d64, _, _ = d_eff_fp64(OracleSolve(live[None], kind="binary"), rtol=1e-11)
    np.testing.assert_allclose(s.D_eff[0], d64[0], rtol=1e-8)
    assert abs(s.D_eff[1]) < 1e-12 * abs(s.D_eff[0])
