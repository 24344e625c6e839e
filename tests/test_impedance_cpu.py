"""CPU tests of the impedance (tau_e) path: the complex128 oracle against the reference's own
outputs (tests/golden/impedance_outputs.npz, made by make_golden.py from
taufactor/electrode.py:160-402), the host's factor table against numpy's and torch's complex
reciprocal, and the C ABI's argument checks (no kernel launches)."""
import os

import numpy as np
import pytest
import torch

from cases import IMPEDANCE_CASES
from oracle import impedance as oi
from taufactor_gb300 import _capi
from taufactor_gb300.impedance import compute_impedance, factor_table

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def imp_golden():
    return np.load(os.path.join(HERE, "golden", "impedance_outputs.npz"))


def _same(a, b):
    """Bitwise equal up to the sign of zero, NaN equal to NaN."""
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("name", sorted(IMPEDANCE_CASES))
def test_impedance_oracle_matches_reference(name, imp_golden):
    periodic, make, kw, solve_kw, _src = IMPEDANCE_CASES[name]
    st = oi.setup(make(), periodic=periodic, **kw)
    g = lambda k: imp_golden[f"{name}/{k}"]  # noqa: E731
    assert np.array_equal(st["vol_x"], g("vol_x"))
    assert np.array_equal(st["a_x"], g("a_x"))
    assert st["freq_0"] == g("freq_0")
    assert np.array_equal(st["frequency"], g("frequency"))
    assert np.array_equal(st["Z_mean"], g("Z_mean"))
    with np.errstate(all="ignore"):
        r = oi.solve(st, **solve_kw)
    assert r["sum_iter"] == int(g("sum_iter"))
    assert r["converged_freq"] == g("converged_freq").tolist()
    # the half-sweeps are the reference's arithmetic: the field is bit for bit the same
    assert _same(r["field"].real, g("field").real) and _same(r["field"].imag, g("field").imag)
    taus = np.array([float(np.asarray(t)[0]) for t in r["taus"]])
    ref = g("taus")
    fin = np.isfinite(ref) & (ref != 0)
    assert np.array_equal(np.isfinite(taus), np.isfinite(ref))
    # layer means are reduced in another order than torch's: last-bit differences only
    assert np.allclose(taus[fin], ref[fin], rtol=1e-12, atol=0)
    imp = np.array(r["impedance"], dtype=np.complex128)
    ok = np.isfinite(g("impedance"))
    assert np.allclose(imp[ok], g("impedance")[ok], rtol=1e-12, atol=0)


def test_impedance_known_answers_through_oracle():
    """tests/test_taufactor.py:253-267: tau_e of the dead-end and through-pore strips."""
    from cases import _imp_deadend, _imp_throughpore

    for make, expect in ((_imp_deadend, 0.594), (_imp_throughpore, 0.986)):
        r = oi.solve(oi.setup(make()))
        assert np.around(r["tau"], 3) == expect


def test_factor_table_is_smith_division():
    """The host's table is numpy's complex128 1 / (nn + i frc nr) (Smith's division) bit for bit,
    and within 2 ulp of torch's (nn + nr * 1j * frc) ** -1 (electrode.py:297), whose CPU kernels
    round differently per instruction set for large frc * nr (equal for the tau_e frequencies)."""
    nn = torch.arange(8, dtype=torch.float64)[:, None].expand(8, 7)
    nr = torch.arange(7, dtype=torch.float64)[None, :].expand(8, 7)
    for frc in (2.34375e-4, 1.171875e-4, 7.8e-5, 0.5, 3.0, 17.25, 1e-9, 123.456):
        t = ((nn + nr * 1j * frc) ** -1).numpy()
        mine = factor_table(frc)
        assert mine[0] == 0
        for a in range(8):
            for b in range(7):
                if a + b == 0:
                    continue
                z = mine[a + 8 * b]
                assert z == np.complex128(1.0) / np.complex128(complex(a, b * frc)), (frc, a, b)
                assert abs(z - t[a, b]) <= 4.5e-16 * abs(z), (frc, a, b)
        assert np.array_equal(mine, oi.factor_table(frc))


def test_compute_impedance_matches_oracle():
    R = np.linspace(1.0, 2.0, 9)
    Cc = np.linspace(0.1, 0.3, 9)
    f = np.array([1e-3, 2e-2, 0.5])
    assert np.array_equal(compute_impedance(R, Cc, f), oi.compute_impedance(R, Cc, f))


def test_impedance_entry_points_reject_bad_arguments_without_launching():
    if not os.path.exists(_capi.lib_path()):
        from taufactor_gb300.build import build

        build()
    lib = _capi.load()
    n0 = lib.tf_launch_count()
    assert lib.tf_impedance_pack(0, 4, 4, 0, 16, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_impedance_pack(4, 4, 4, 0, None, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_impedance_fill(1, 4, 4, 4, 16, 16, 2.0, 8, None) == _capi.TF_ERR_ARG  # misaligned field
    assert lib.tf_impedance_fill(0, 4, 4, 4, 16, 16, 2.0, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_impedance_sweep(1, 4, 4, 4, 0, 16, 16, 24, None, 1.5, 0, 1, None) == _capi.TF_ERR_ARG
    assert lib.tf_impedance_sweep(1, 4, 4, 4, 0, 16, 16, 16, None, 1.5, 0, -1, None) == _capi.TF_ERR_ARG
    assert lib.tf_impedance_sweep(70000, 4, 4, 4, 0, 16, 16, 16, None, 1.5, 0, 1, None) == _capi.TF_ERR_ARG
    assert lib.tf_impedance_metrics(1, 4, 4, 4, None, 1.0, 16, 16, 16, None) == _capi.TF_ERR_ARG
    assert lib.tf_launch_count() == n0
