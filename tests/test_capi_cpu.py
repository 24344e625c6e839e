"""CPU tests of the C ABI and of the host-side logic (no kernel launches)."""
import ctypes as C
import re
import warnings

import numpy as np
import pytest

from taufactor_gb300 import _capi
from taufactor_gb300.solvers import (AnisotropicSolver, MultiPhaseSolver, Solver, anisotropic_divisors,
                                     harmonic_face)


@pytest.fixture(scope="module")
def lib():
    import os

    if not os.path.exists(_capi.lib_path()):
        from taufactor_gb300.build import build

        build()
    return _capi.load()


def test_header_declares_exactly_the_exports(lib):
    import os

    with open(os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "taufactor_gb300.h")) as f:
        hdr = f.read()
    declared = set(re.findall(r"\b(tf_[a-z_0-9]+)\s*\(", hdr))
    assert declared == set(_capi.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_version_and_status(lib):
    assert b"sm_103a" in lib.tf_version()
    assert lib.tf_status_string(0) == b"ok"
    assert lib.tf_status_string(_capi.TF_ERR_TIMEOUT) == b"device wait timed out"


def test_geometry(lib):
    g = _capi.TfGeom()
    assert lib.tf_geometry(2, 10, 9, 13, 0, C.byref(g)) == 0
    assert (g.batch, g.nx, g.ny, g.nz) == (2, 10, 9, 13)
    assert g.yp == 9 + 2 * g.halo_y
    assert g.zh % 4 == 0 and g.zh >= 7 + 2 * g.halo_j
    assert g.zhc % 16 == 0 and g.zhc >= g.zh
    assert g.field_elems == 2 * 10 * g.yp * 2 * g.zh
    assert g.code_bytes == 2 * 10 * g.yp * 2 * g.zhc
    assert g.tiled == 1
    assert lib.tf_geometry(1, 10, 9, 13, _capi.TF_PERIODIC_Y, C.byref(g)) == 0 and g.tiled == 0
    assert lib.tf_geometry(1, 10, 10, 16, 3, C.byref(g)) == 0 and g.tiled == 1
    assert lib.tf_geometry(0, 10, 9, 13, 0, C.byref(g)) == _capi.TF_ERR_ARG


def test_entry_points_reject_bad_arguments_without_launching(lib):
    g = _capi.TfGeom()
    lib.tf_geometry(1, 8, 8, 8, 0, C.byref(g))
    op = _capi.TfOperator()
    op.omega = 1.5
    n0 = lib.tf_launch_count()
    assert lib.tf_pack(C.byref(g), C.byref(op), None, None, None, None, None) == _capi.TF_ERR_ARG
    res = C.c_int(0)
    assert lib.tf_advance(C.byref(g), C.byref(op), None, None, None, 0, 4, None, C.byref(res), None) == \
        _capi.TF_ERR_ARG
    bad = _capi.TfGeom.from_buffer_copy(g)
    bad.zh = 3
    assert lib.tf_layer_sums(C.byref(bad), C.byref(op), 16, 16, 16, 16, None) == _capi.TF_ERR_ARG
    op.kind = 7
    assert lib.tf_unpack(C.byref(g), C.byref(op), 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_anchored_phase(1, 4, 4, 4, 0, None, 16, 16, 16, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_anchored_phase(1, 0, 4, 4, 0, 16, 16, 16, 16, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_stats(0, 4, 4, 4, 16, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_stats(1, 4, 4, 4, None, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_stats(2, 40000, 4, 4, 16, 16, 16, None) == _capi.TF_ERR_UNSUPPORTED  # > 65535 planes
    assert lib.tf_batch_advance_tile(16, 16, 4, 16, 0, 3, None) == _capi.TF_ERR_ARG  # no tile class 3
    assert lib.tf_batch_advance_rhs_tile(16, 16, 4, 16, 0, -1, None) == _capi.TF_ERR_ARG
    assert lib.tf_launch_count() == n0
    with pytest.raises(ValueError):
        _capi.check(_capi.TF_ERR_ARG, "x")
    with pytest.raises(_capi.TfError):
        _capi.check(_capi.TF_ERR_CUDA, "x")


def test_static_scratch_entry_point_refuses_without_launching(lib):
    """tf_batch_converge_static (the allocation-free convergence step) refuses missing state
    pointers, arena lengths beyond its fixed array and a descriptor table that tf_batch_describe
    never built, all before it launches anything."""
    st = _capi.TfBatchState(*([16] * 9))
    n0 = lib.tf_launch_count()
    assert lib.tf_batch_converge_static(None, 16, 1, 1, 10, 10, st, 1e-2, 0, 0, None) == _capi.TF_ERR_ARG
    assert lib.tf_batch_converge_static(16, None, 1, 1, 10, 10, st, 1e-2, 0, 0, None) == _capi.TF_ERR_ARG
    assert lib.tf_batch_converge_static(16, 16, 0, 1, 10, 10, st, 1e-2, 0, 0, None) == _capi.TF_ERR_ARG
    empty = _capi.TfBatchState(*([16] * 8 + [0]))
    assert lib.tf_batch_converge_static(16, 16, 1, 1, 10, 10, empty, 1e-2, 0, 0, None) == _capi.TF_ERR_ARG
    assert lib.tf_batch_converge_static(16, 16, 1, 1, 65537, 10, st, 1e-2, 0, 0, None) == _capi.TF_ERR_UNSUPPORTED
    assert lib.tf_batch_converge_static(16, 16, 1, 1, 10, 65537, st, 1e-2, 0, 0, None) == _capi.TF_ERR_UNSUPPORTED
    # a table address tf_batch_describe never filled (no device here either): refused
    assert lib.tf_batch_converge_static(4096, 16, 1, 1, 10, 10, st, 1e-2, 0, 0, None) == _capi.TF_ERR_ARG
    assert lib.tf_launch_count() == n0


def test_anisotropic_divisors_match_reference_order():
    """LUT entries equal the reference's rolled sums on a volume exercising every pattern."""
    from oracle.sor import neighbour_counts

    ky, kz = (1.0 / 1.3) ** 2, (1.0 / 0.7) ** 2
    lut = anisotropic_divisors(ky, kz)
    rng = np.random.default_rng(3)
    mask = (rng.random((1, 7, 9, 11)) < 0.6).astype(np.float32)
    nn = neighbour_counts(mask, False, (1.0, ky, kz))
    p = np.pad(mask[0], 1)
    p[0] = 2
    p[-1] = 2
    for x in range(7):
        for y in range(9):
            for z in range(11):
                if mask[0, x, y, z] == 0:
                    continue
                xm, xp = int(p[x, y + 1, z + 1]), int(p[x + 2, y + 1, z + 1])
                ym, yp = int(p[x + 1, y, z + 1]), int(p[x + 1, y + 2, z + 1])
                zm, zp = int(p[x + 1, y + 1, z]), int(p[x + 1, y + 1, z + 2])
                idx = 1 + xm + 3 * xp + 9 * ym + 18 * yp + 36 * zm + 72 * zp
                assert lut[idx] == nn[0, x, y, z] or (np.isinf(lut[idx]) and np.isinf(nn[0, x, y, z]))


def test_harmonic_face_matches_reference_formula():
    from oracle.sor import harmonic_mean

    vals = np.array([0.0, 0.1, 0.5, 1.0, 2.0, 0.3, 1e-3], dtype=np.float32)
    a, b = np.meshgrid(vals, vals, indexing="ij")
    hm = harmonic_mean(a, b)
    for i in range(len(vals)):
        for j in range(len(vals)):
            assert harmonic_face(vals[i], vals[j]) == hm[i, j]


def test_validation_errors_match_reference():
    with pytest.raises(TypeError):
        Solver([[0, 1], [1, 0]])
    with pytest.raises(ValueError, match="Input image must only contain 0s and 1s"):
        Solver(np.full((4, 4, 4), 2))
    with pytest.raises(ValueError, match=r"expected \[B, X, Y, Z\]"):
        Solver(np.ones((1, 1, 2, 2, 2)))
    with pytest.raises(ValueError):
        MultiPhaseSolver(np.zeros((6, 6, 6)), {0: 1.0, 1: -0.1})
    with pytest.raises(TypeError):
        MultiPhaseSolver(np.zeros((6, 6, 6)), [1, 2])
    with pytest.raises(TypeError):
        MultiPhaseSolver(np.zeros((6, 6, 6)), {"a": 1.0})
    with pytest.raises(ValueError, match="spacing"):
        AnisotropicSolver(np.ones((4, 4, 4)), (1, 2))


def test_no_cpu_fallback():
    """The reference falls back to the CPU; this package refuses."""
    with pytest.raises(RuntimeError, match="CUDA"):
        Solver(np.ones((4, 4, 4)), device="cpu")


def test_multiphase_missing_label_warning_before_device():
    img = np.zeros((6, 6, 6))
    img[:, :, 3:] = 2
    ds = {0: 1.0}
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        try:
            MultiPhaseSolver(img, ds, device="cpu")
        except RuntimeError:
            pass
    assert any("assuming these phases are isolating." in str(x.message) for x in w)
    assert ds[2] == 0.0


def test_multigrid_level_dims():
    """The multigrid hierarchy's shapes: extents >= 4 halve (rounding up), smaller ones stay,
    periodic extents only while the half is even; the coarsest level cannot be halved again."""
    from taufactor_gb300.multigrid import level_dims

    assert level_dims((768, 768, 768), 0) == [(768,) * 3, (384,) * 3, (192,) * 3, (96,) * 3, (48,) * 3,
                                              (24,) * 3, (12,) * 3, (6,) * 3, (3,) * 3]
    assert level_dims((40, 3, 70), 0) == [(40, 3, 70), (20, 3, 35), (10, 3, 18), (5, 3, 9), (3, 3, 5), (3, 3, 3)]
    assert level_dims((3, 3, 3), 0) == [(3, 3, 3)]
    per = level_dims((320, 320, 320), 3)
    assert per[-1] == (3, 10, 10)
    assert all(d[1] % 2 == 0 and d[2] % 2 == 0 for d in per)
    assert level_dims((14, 12, 16), 3) == [(14, 12, 16), (7, 6, 8), (4, 6, 4), (2, 6, 2)]
    for dims, p in [((100, 37, 9), 0), ((64, 48, 80), 3), ((5, 200, 6), 1)]:
        lv = level_dims(dims, p)
        for f, c in zip(lv, lv[1:]):
            assert all(cc in (ff, (ff + 1) // 2) for ff, cc in zip(f, c))
        assert level_dims(lv[-1], p) == [lv[-1]]


def test_refinement_keeps_the_percolation_verdict():
    """A volume the float32 solve declared non-percolating (tau 0 or inf) keeps tau = inf,
    D_eff = 0 and tau_x = 0 after the FP64 correction; the others keep their refined values."""
    from types import SimpleNamespace

    from taufactor_gb300.solvers import keep_non_percolating

    s = SimpleNamespace(tau=np.array([1.9, 3.2e15, 2.5]), D_eff=np.array([0.4, 1e-17, 0.3]),
                        tau_x=np.ones((3, 4)))
    keep_non_percolating(s, np.array([1.91, np.inf, 0.0]))
    assert s.tau[0] == 1.9 and np.isinf(s.tau[1]) and np.isinf(s.tau[2])
    assert s.D_eff.tolist() == [0.4, 0.0, 0.0]
    assert s.tau_x[0].tolist() == [1.0] * 4 and not s.tau_x[1:].any()
    t = SimpleNamespace(tau=np.array([1.0]), D_eff=np.array([0.5]), tau_x=None)
    keep_non_percolating(t, None)
    assert t.tau[0] == 1.0 and t.D_eff[0] == 0.5


def test_multigrid_and_kappa_entry_points_refuse_bad_arguments(lib):
    """The multigrid, float64-face and fused-sweep entry points check their arguments before
    any launch: levels that are not a coarsening of each other, missing or misaligned buffers,
    one field passed as both ping-pong buffers, a second dot product without its partner."""
    f, c, wrong = _capi.TfGeom(), _capi.TfGeom(), _capi.TfGeom()
    lib.tf_geometry(1, 16, 12, 10, 0, C.byref(f))
    lib.tf_geometry(1, 8, 6, 5, 0, C.byref(c))
    lib.tf_geometry(1, 8, 5, 5, 0, C.byref(wrong))  # 12 -> 5 is no halving
    op = _capi.TfOperator()
    op.omega = 1.0
    n0 = lib.tf_launch_count()
    P = 4096  # a 16-byte aligned stand-in pointer; nothing is dereferenced on refusal
    assert lib.tf_mg_coarsen(C.byref(f), P, P, P, C.byref(wrong), P, P, P, P, 0, 0.5, None) == _capi.TF_ERR_ARG
    assert lib.tf_mg_coarsen(C.byref(f), P, P, P, C.byref(c), P, P, P, P, 0, 0.0, None) == _capi.TF_ERR_ARG
    assert lib.tf_mg_coarsen(C.byref(f), None, P, P, C.byref(c), P, P, P, P, 0, 0.5, None) == _capi.TF_ERR_ARG
    assert lib.tf_mg_restrict(C.byref(f), P, P, P, P, P, P, C.byref(wrong), P, None) == _capi.TF_ERR_ARG
    assert lib.tf_mg_prolong(C.byref(wrong), P, C.byref(f), P, 0, None) == _capi.TF_ERR_ARG
    assert lib.tf_mg_apply(C.byref(f), P + 4, P, P, P, P, P, None) == _capi.TF_ERR_ARG  # misaligned
    assert lib.tf_mg_dot(C.byref(f), P, P, P, None, P, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_pcg_update_xr(C.byref(f), P, P, P, None, P, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_pcg_update_p(C.byref(f), P + 8, P, P, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_kappa_faces_f64(C.byref(f), None, P, P, P, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_kappa_residual_faces_f64(C.byref(f), C.byref(op), P, P, P, P, None, None, P, P, P, None) == \
        _capi.TF_ERR_ARG
    res = C.c_int(0)
    assert lib.tf_kappa_advance_fused(C.byref(f), C.byref(op), P, P, P, P, P, P, None, 0, 4, None, C.byref(res),
                                      None) == _capi.TF_ERR_ARG  # the same buffer twice
    assert lib.tf_kappa_advance_fused(C.byref(f), C.byref(op), P, P + 16, P, P, P, P, P + 4, 0, 4, None,
                                      C.byref(res), None) == _capi.TF_ERR_ARG  # misaligned rhs
    assert lib.tf_refresh_ghosts(C.byref(f), 3, None, None) == _capi.TF_ERR_ARG
    assert lib.tf_refresh_ghosts(C.byref(f), 0, P, None) == _capi.TF_OK  # nothing to do, no launch
    assert lib.tf_launch_count() == n0


def test_label_map_and_sums_refuse_bad_arguments(lib):
    """tf_label_map and tf_label_sums check their arguments before any launch."""
    n0 = lib.tf_launch_count()
    P = 1 << 20  # a non-null address that is never dereferenced: every call below is refused
    assert lib.tf_label_map(None, 10, P, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_map(P, 0, P, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_map(P, 10, P, None, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_sums(1, 4, 4, 4, P, P, P, 0, P, None) == _capi.TF_ERR_ARG  # no slots
    assert lib.tf_label_sums(1, 4, 4, 4, P, P, P, 257, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_sums(0, 4, 4, 4, P, P, P, 3, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_label_sums(1, 4, 4, 4, P, None, P, 3, P, None) == _capi.TF_ERR_ARG
    assert lib.tf_launch_count() == n0


def test_default_kernel_configuration_per_operator_kind():
    """Untuned solvers start from the measured best tile and fused depth of their kind: the
    binary kind on 16 x 128 tiles when z spans a tile, multiphase 3 half-sweeps per launch,
    the others 4 on 16 x 64 tiles."""
    from types import SimpleNamespace

    from taufactor_gb300.autotune import default_config

    def fake(kind, nz):
        return SimpleNamespace(_op=SimpleNamespace(kind=kind), Nz=nz)

    assert default_config(fake(_capi.TF_KIND_BINARY, 256)) == (1, 4)
    assert default_config(fake(_capi.TF_KIND_BINARY, 64)) == (0, 4)
    assert default_config(fake(_capi.TF_KIND_MULTIPHASE, 320)) == (0, 3)
    assert default_config(fake(_capi.TF_KIND_ELECTRODE, 256)) == (0, 4)
    assert default_config(fake(_capi.TF_KIND_ANISOTROPIC, 256)) == (0, 4)
