"""GPU tests of the per-voxel conductivity operator and its adjoint gradients.

Bars: with kappa = D[label] the half-sweeps equal MultiPhaseSolver's bit for bit; the refined
D_eff is within 1e-9 of the FP64 oracle (float32 and float64 face coefficients); dD_eff/dkappa is
within 1e-6 of the FP64 oracle's adjoint gradient, within 1e-4 (target 1e-3) of central finite
differences (h = 1e-3) and satisfies Euler's identity sum(kappa dD/dkappa) = D_eff (D_eff is
homogeneous of degree 1 in kappa); the adjoint costs at most 3x the forward solve.
"""
import numpy as np
import pytest
import torch

from cases import random_labels
from oracle.fp64 import adjoint_gradient_fp64, d_eff_fp64
from oracle.sor import OracleSolve

pytestmark = pytest.mark.gpu

import taufactor_gb300 as tg  # noqa: E402


def _kappa(shape, seed, lo=0.05):
    return (lo + np.random.default_rng(seed).random(shape)).astype(np.float32)


@pytest.mark.parametrize("periodic", [False, True])
def test_kappa_from_labels_equals_multiphase_bitwise(periodic):
    lab = random_labels((14, 12, 16), 61)
    ds = {0: 0.0, 1: 1.0, 2: 0.1}
    kap = np.vectorize(lambda v: ds[int(v)])(lab).astype(np.float32)
    o = OracleSolve(lab, kind="periodic_multiphase" if periodic else "multiphase", diffusivities=ds)
    s = tg.KappaSolver(kap, periodic=periodic)
    for n in (3, 8, 13):
        s._advance(n, s._c)
        s.iter += n
        o.half_sweep(n)
        got = s.field().cpu().numpy()[:, :, 1:-1, 1:-1]
        assert np.array_equal(got, o.field[:, :, 1:-1, 1:-1]), n


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("shape", [(1, 9, 12, 18), (2, 7, 10, 13), (1, 5, 16, 40)])
def test_packed_face_sweeps_equal_direct_sweeps(shape, periodic):
    """tf_kappa_advance_faces (faces packed once) gives tf_kappa_advance's bits, with and without
    a right-hand side, on kappa fields with zeros, odd z-lengths and partial float4 groups."""
    import ctypes as C

    from taufactor_gb300._capi import TfOperator, check

    if periodic and (shape[2] % 2 or shape[3] % 2):
        pytest.skip("periodic faces of odd size run the reference's diverging iteration")
    rng = np.random.default_rng(sum(shape))
    kap = (rng.random(shape) * (rng.random(shape) > 0.2)).astype(np.float32)
    s = tg.KappaSolver(kap, periodic=periodic)
    lib, g, st = s._lib, s._geom, s._stream()
    a = s._c.clone()
    b = s._c.clone()
    rhs = (0.01 * torch.randn(g.field_elems, device="cuda")).float()
    rhs[s._ks == 0] = 0
    for n, r, c0 in ((3, None, 0), (4, rhs, 1), (5, None, 1)):
        rp = r.data_ptr() if r is not None else None
        check(lib.tf_kappa_advance(C.byref(g), C.byref(s._op), a.data_ptr(), s._ks.data_ptr(), rp, c0, n, st),
              "tf_kappa_advance")
        check(lib.tf_kappa_advance_faces(C.byref(g), C.byref(s._op), b.data_ptr(), s._fx.data_ptr(),
                                         s._fy.data_ptr(), s._fz.data_ptr(), s._dv.data_ptr(), rp, c0, n, st),
              "tf_kappa_advance_faces")
        torch.cuda.synchronize()
        assert torch.equal(a.view(torch.int32), b.view(torch.int32)), n


@pytest.mark.parametrize("coefficients", ["f32", "f64"])
@pytest.mark.parametrize("kind", ["kappa", "periodic_kappa"])
def test_refined_d_eff_and_gradient_match_fp64_oracle(kind, coefficients):
    kap = _kappa((1, 14, 12, 16), 62)
    s = tg.KappaSolver(kap, periodic=kind == "periodic_kappa", coefficients=coefficients)
    s.solve(conv_crit=1e-3, refine={"tol": 1e-12})
    o = OracleSolve(kap, kind=kind)
    d64, _, _ = d_eff_fp64(o, rtol=1e-12, coefficients=coefficients)
    np.testing.assert_allclose(s.D_eff, d64, rtol=1e-9)
    g = s.gradient(tol=1e-12).cpu().numpy()
    assert s.adjoint_history[-1] < 1e-12
    gref = adjoint_gradient_fp64(o, rtol=1e-12, coefficients=coefficients)
    scale = np.abs(gref).max()
    np.testing.assert_allclose(g, gref, rtol=1e-6, atol=1e-8 * scale)


def test_gradient_matches_central_finite_differences():
    kap = _kappa((16, 14, 18), 63)
    s = tg.KappaSolver(kap)
    s.solve(conv_crit=1e-3, refine={"tol": 1e-13})
    g = s.gradient(tol=1e-13).cpu().numpy()[0]
    rng = np.random.default_rng(64)
    errs = []
    for _ in range(8):
        i = tuple(int(rng.integers(0, n)) for n in kap.shape)
        kp, km = kap.copy(), kap.copy()
        kp[i] += np.float32(1e-3)
        km[i] -= np.float32(1e-3)
        dp = tg.KappaSolver(kp)
        dp.warm_start(s)
        dp.solve(conv_crit=1e-3, refine={"tol": 1e-13})
        dm = tg.KappaSolver(km)
        dm.warm_start(s)
        dm.solve(conv_crit=1e-3, refine={"tol": 1e-13})
        fd = (dp.D_eff[0] - dm.D_eff[0]) / (float(kp[i]) - float(km[i]))
        errs.append(abs(fd - g[i]) / abs(fd))
    assert max(errs) < 1e-4, errs


@pytest.mark.parametrize("periodic", [False, True])
def test_gradient_euler_identity(periodic):
    """D_eff(s kappa) = s D_eff(kappa), so sum(kappa * dD_eff/dkappa) = D_eff at any size."""
    from scipy.ndimage import gaussian_filter

    logits = gaussian_filter(np.random.default_rng(67).standard_normal((48, 40, 56)), 2.0)
    kap = (1.0 / (1.0 + np.exp(-2.0 * logits))).astype(np.float32)
    s = tg.KappaSolver(kap, periodic=periodic)
    s.solve(conv_crit=1e-3, refine={"tol": 1e-13})
    g = s.gradient(tol=1e-13)
    d = float(s.D_eff[0])
    assert abs(float((s.kappa.double() * g).sum()) - d) / d < 1e-9


def test_autograd_function_and_cost_ratio():
    kap = torch.from_numpy(_kappa((64, 64, 64), 65)).cuda().requires_grad_(True)
    d = tg.d_eff(kap)
    d.backward()
    s = tg.KappaSolver(kap.detach())
    s.solve(conv_crit=1e-3, refine={"tol": 1e-11})
    g = s.gradient(tol=1e-11)[0].float()
    torch.testing.assert_close(kap.grad, g, rtol=1e-6, atol=1e-12)
    fwd = s.walltime
    adj = s.timings["adjoint_s"]
    assert adj <= 3 * fwd, (adj, fwd)


def test_multiphase_phase_gradients_match_finite_differences():
    lab = random_labels((14, 12, 16), 66)
    ds = {0: 0.2, 1: 1.0, 2: 0.5}
    s = tg.MultiPhaseSolver(lab, dict(ds))
    s.solve(verbose=False, conv_crit=1e-3)
    grads = s.phase_gradients(tol=1e-13)
    # the float32 loop before the correction (method "sor") reaches the same corrected field
    grads_sor = s.phase_gradients(tol=1e-13, method="sor")
    for p in grads:
        np.testing.assert_allclose(grads_sor[p], grads[p], rtol=1e-8, atol=1e-12)
    for p in (0, 2):
        h = 1e-3
        up, dn = dict(ds), dict(ds)
        up[p] += h
        dn[p] -= h
        a = tg.MultiPhaseSolver(lab, up)
        a.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-13})
        b = tg.MultiPhaseSolver(lab, dn)
        b.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-13})
        hp = float(np.float32(up[p])) - float(np.float32(dn[p]))
        fd = (a.D_eff[0] - b.D_eff[0]) / hp
        assert abs(fd - grads[p][0]) / abs(fd) < 1e-3, (p, fd, grads[p][0])


def test_phase_gradients_device_labels_match_host_labels():
    """uint8 labels take the device path (tf_label_map, tf_label_sums); the same labels as int64
    take the host path: the same kappa field, so the same solve, and per-label sums equal to
    float64 rounding."""
    lab = random_labels((2, 12, 10, 14), 67)
    ds = {0: 0.3, 1: 1.0, 2: 0.05}
    a = tg.MultiPhaseSolver(lab, dict(ds))
    b = tg.MultiPhaseSolver(lab.astype(np.int64), dict(ds))
    ga = a.phase_gradients(tol=1e-12)
    gb = b.phase_gradients(tol=1e-12)
    assert torch.equal(a.kappa_solver.kappa, b.kappa_solver.kappa)
    for p in ds:
        np.testing.assert_allclose(ga[p], gb[p], rtol=1e-12, atol=1e-15)


def test_kappa_set_up_statistics_and_input_check():
    """vol_x and D_mean come from one device pass (tf_kappa_stats) and match the host
    computation; negative, infinite and NaN conductivities are refused."""
    import taufactor_gb300 as tg

    rng = np.random.default_rng(61)
    k = rng.random((2, 9, 11, 13)).astype(np.float32)
    k[k < 0.3] = 0.0
    s = tg.KappaSolver(k)
    assert np.array_equal(s.vol_x, (k > 0).reshape(2, 9, -1).sum(axis=2) / float(11 * 13))
    np.testing.assert_allclose(s.D_mean, k.astype(np.float64).mean(axis=(1, 2, 3)), rtol=1e-14, atol=0)
    for v in (-0.5, np.inf, np.nan):
        bad = k.copy()
        bad[1, 4, 5, 6] = v
        with pytest.raises(ValueError, match="finite and >= 0"):
            tg.KappaSolver(bad)


def test_design_loop_warm_started_steps():
    """The gradient-driven design loop's building blocks on a small volume: three Adam steps on
    the logits of kappa = sigmoid(logits), each a forward solve warm-started from the previous
    step's field and refined to 1e-10, and an adjoint solve started from the previous adjoint
    field (lam0). Every step reaches its residuals and Euler's identity, and warm starts need no
    more outer steps than the cold first step; the last gradient matches a directional central
    difference (h = 1e-3) to 1e-6."""
    from scipy.ndimage import gaussian_filter

    logits0 = gaussian_filter(np.random.default_rng(77).standard_normal((40, 36, 32)).astype(np.float32), 3.0)
    logits = torch.from_numpy(logits0).cuda().requires_grad_(True)
    opt = torch.optim.Adam([logits], lr=0.05, maximize=True)
    prev = None
    outers = []
    for _ in range(3):
        with torch.no_grad():
            kap = torch.sigmoid(logits).float().contiguous()
        s = tg.KappaSolver(kap)
        if prev is not None:
            s.warm_start(prev)
        s.solve(conv_crit=1e-3, refine={"tol": 1e-10, "max_outer": 40})
        g = s.gradient(tol=1e-10, max_outer=40, lam0=prev.lam if prev is not None else None)[0]
        assert s.residual_history[-1] < 1e-10 and s.adjoint_history[-1] < 1e-10
        d = float(s.D_eff[0])
        assert abs(float((s.kappa[0].double() * g).sum()) - d) / d < 1e-9
        outers.append(len(s.adjoint_history))
        with torch.no_grad():
            kk = kap.double()
            logits.grad = ((g - 0.5 / kap.numel()) * kk * (1.0 - kk)).float()
        opt.step()
        prev = s
    assert max(outers[1:]) <= outers[0]
    kap = prev.kappa[0]
    direc = torch.sign(g).float()

    def deff(kk):
        t = tg.KappaSolver(kk.contiguous())
        t.warm_start(prev)
        t.solve(conv_crit=1e-3, refine={"tol": 1e-13, "max_outer": 60})
        return float(t.D_eff[0])

    kp, km = (kap + 1e-3 * direc).float(), (kap - 1e-3 * direc).float()
    fd = (deff(kp) - deff(km)) / 2.0
    ad = float((g * ((kp.double() - km.double()) / 2.0)).sum())
    assert abs(fd - ad) / abs(fd) < 1e-6


@pytest.mark.parametrize("k_max", [1, 3, 4])
@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("shape", [(1, 9, 12, 18), (2, 37, 20, 40), (1, 40, 36, 130), (2, 150, 16, 64)])
def test_fused_face_sweeps_equal_single_sweeps(shape, periodic, k_max):
    """tf_kappa_advance_fused (K half-sweeps per register-streaming launch, faces read per group)
    gives tf_kappa_advance_faces's bits: kappa with zeros, partial tiles in y and z, x-chunked
    columns, periodic ghost bands, with and without a right-hand side, both colour starts."""
    import ctypes as C

    from taufactor_gb300._capi import TfOperator, check

    rng = np.random.default_rng(sum(shape) + k_max)
    kap = (rng.random(shape) * (rng.random(shape) > 0.2)).astype(np.float32)
    s = tg.KappaSolver(kap, periodic=periodic)
    lib, g, st = s._lib, s._geom, s._stream()
    op = TfOperator.from_buffer_copy(s._op)
    op.k_max = k_max
    a = s._c.clone()
    fa, fb = s._c.clone(), torch.zeros_like(s._c)
    rhs = (0.01 * torch.randn(g.field_elems, device="cuda")).float()
    rhs[s._ks == 0] = 0
    check(lib.tf_refresh_ghosts(C.byref(g), s._op.periodic, rhs.data_ptr(), st), "tf_refresh_ghosts")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    faces = [s._fx.data_ptr(), s._fy.data_ptr(), s._fz.data_ptr(), s._dv.data_ptr()]
    for n, r, c0 in ((4, None, 0), (7, rhs, 1), (5, None, 1), (8, rhs, 0)):
        rp = r.data_ptr() if r is not None else None
        check(lib.tf_kappa_advance_faces(C.byref(g), C.byref(op), a.data_ptr(), *faces, rp, c0, n, st),
              "tf_kappa_advance_faces")
        in_b = C.c_int(0)
        check(lib.tf_kappa_advance_fused(C.byref(g), C.byref(op), fa.data_ptr(), fb.data_ptr(), *faces, rp, c0, n,
                                         err.data_ptr(), C.byref(in_b), st), "tf_kappa_advance_fused")
        if in_b.value:
            fa, fb = fb, fa
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        m = torch.zeros(g.field_elems, dtype=torch.bool, device="cuda")
        lay_row, lay_plane = 2 * g.zh, 2 * g.zh * g.yp
        b_, x_, y_, z_ = np.meshgrid(np.arange(s.batch_size), np.arange(s.Nx), np.arange(s.Ny), np.arange(s.Nz),
                                     indexing="ij")
        idx = (b_ * s.Nx + x_) * lay_plane + (y_ + 4) * lay_row + (z_ & 1) * g.zh + 4 + (z_ >> 1)
        m[torch.from_numpy(idx.ravel()).cuda()] = True
        assert torch.equal(a[m].view(torch.int32), fa[m].view(torch.int32)), n
