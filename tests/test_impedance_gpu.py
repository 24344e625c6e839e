"""GPU parity tests of the impedance (tau_e) solvers (taufactor/electrode.py:160-402): the sm_103a
path against the reference's own outputs, against the complex128 oracle bit for bit, against a
direct sparse solve, and the reference's known answers (tests/test_taufactor.py:253-267)."""
import contextlib
import io
import os

import numpy as np
import pytest

from cases import IMPEDANCE_CASES, _imp_blob, _imp_deadend, _imp_throughpore

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def imp_golden():
    return np.load(os.path.join(HERE, "golden", "impedance_outputs.npz"))


def _solver(periodic):
    import taufactor_gb300 as tg

    return tg.PeriodicImpedanceSolver if periodic else tg.ImpedanceSolver


def _quiet_solve(s, **kw):
    with contextlib.redirect_stdout(io.StringIO()) as out, np.errstate(all="ignore"):
        s.solve(verbose=False, **kw)
    return out.getvalue()


def _close_or_same(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    fa, fb = np.isfinite(a), np.isfinite(b)
    if not np.array_equal(fa, fb) or not np.array_equal(np.isnan(a), np.isnan(b)):
        return False
    if not np.array_equal(a[~fa & ~np.isnan(a)], b[~fb & ~np.isnan(b)]):
        return False
    return bool(np.all(np.abs(a[fa] - b[fb]) <= rtol * np.abs(b[fb]) + 1e-300))


@pytest.mark.parametrize("name", sorted(IMPEDANCE_CASES))
def test_impedance_matches_reference_goldens(name, imp_golden):
    periodic, make, kw, solve_kw, _src = IMPEDANCE_CASES[name]
    s = _solver(periodic)(make(), device="cuda", **kw)
    g = lambda k: imp_golden[f"{name}/{k}"]  # noqa: E731
    assert np.array_equal(s.vol_x, g("vol_x")) and np.array_equal(s.a_x, g("a_x"))
    assert s.freq_0 == g("freq_0") and np.array_equal(s.frequency, g("frequency"))
    assert np.array_equal(s.Z_mean, g("Z_mean"))
    out = _quiet_solve(s, **solve_kw)
    assert out.startswith("[")  # print(self.taus) (electrode.py:319)
    assert s.sum_iter == int(g("sum_iter"))
    assert s.converged_freq == g("converged_freq").tolist()
    taus = np.array([float(np.asarray(t)[0]) for t in s.taus])
    assert _close_or_same(taus, g("taus"), 1e-9)
    imp = np.array(s.impedance, dtype=np.complex128)
    assert _close_or_same(imp.real, g("impedance").real, 1e-9)
    assert _close_or_same(imp.imag, g("impedance").imag, 1e-9)
    field = s.field.cpu().numpy()[0]
    ref = g("field")
    for part in ("real", "imag"):
        a, b = getattr(field, part), getattr(ref, part)
        fin = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), fin) and np.array_equal(np.isnan(a), np.isnan(b))
        if fin.any():
            scale = np.abs(b[fin]).max()
            assert np.abs(a[fin] - b[fin]).max() <= 1e-9 * scale


@pytest.mark.parametrize("periodic,shape,seed,n_half", [
    (False, (13, 11, 9), 41, 137),
    (True, (12, 9, 11), 42, 137),
    (True, (10, 12, 14), 43, 64),
    (False, (40, 30, 1), 44, 101),
])
def test_impedance_half_sweeps_bitwise_against_oracle(periodic, shape, seed, n_half):
    """n_half half-sweeps from the analytic profile at a high frequency (large frc * nr): the
    device field equals the oracle's bit for bit (up to the sign of zero)."""
    from oracle import impedance as oi

    img = _imp_blob(shape, seed, inert=0.2) if shape[2] > 1 else _imp_blob(shape, seed)
    s = _solver(periodic)(img, device="cuda")
    st = oi.setup(img, periodic=periodic)
    frc = float(st["frequency"][0] * 300.0)
    s.frc = frc
    s.field = s.init_field_internal(s.mask)
    s._set_factor(frc)
    s.iter = 0
    s._advance(n_half)
    got = s.field.cpu().numpy()[0]
    f = oi.init_field(st, frc)
    code = (st["nn"] + 8 * st["nr"]).astype(np.int64)
    code[st["mask"] == 0] = 0
    fac = oi.factor_table(frc)[code]
    cb = oi.chequerboard(st["shape"], s.omega)
    for it in range(n_half):
        oi.half_sweep(f, fac, cb[it % 2], periodic)
    # ghosts included: both copy them before every half-sweep
    assert np.array_equal(got, f)


def test_impedance_known_answers():
    """tests/test_taufactor.py:253-267 on the device."""
    for make, expect in ((_imp_deadend, 0.594), (_imp_throughpore, 0.986)):
        s = _solver(False)(make(), device="cuda")
        _quiet_solve(s)
        assert np.around(s.tau, 3) == expect


def _strip40():
    img = np.zeros((40, 40))
    img[:, 15:25] = 1
    return img


@pytest.mark.parametrize("periodic,make", [
    (True, lambda: _imp_blob((14, 10, 12), 31)),
    (False, _strip40),
])
def test_solve_frequencies_matches_direct_solve(periodic, make):
    from oracle import impedance as oi

    img = make()
    s = _solver(periodic)(img, device="cuda", mode="nyquist")
    st = oi.setup(img, periodic=periodic, mode="nyquist")
    freqs = s.frequency[-6:]  # the low-frequency end, where the sweeps converge
    r = s.solve_frequencies(freqs, conv_crit=1e-6, iter_limit=40000)
    assert r["converged"].all()
    for k, frc in enumerate(freqs):
        z = oi.input_impedance(oi.direct_field(st, frc))
        assert abs(r["impedance"][k] - z) <= 1e-6 * abs(z)
        assert r["tau"][k] == r["impedance"][k].real / s.Z_mean[-1].real


def test_impedance_rejects_batches_and_host_devices():
    import taufactor_gb300 as tg

    with pytest.raises(TypeError):
        tg.ImpedanceSolver(np.ones((2, 4, 4, 4)), device="cuda")
    with pytest.raises(RuntimeError):
        tg.ImpedanceSolver(np.ones((4, 4, 4)), device="cpu")
    s = tg.ImpedanceSolver(_imp_blob((8, 6, 6), 3), device="cuda")
    with pytest.raises(ValueError):
        s.field = np.zeros((1, 10, 8, 8), dtype=np.complex128)
        s._advance(2)
