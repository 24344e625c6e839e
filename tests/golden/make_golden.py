"""Generate ``reference_outputs.npz`` by running the reference package itself.

Usage (needs the reference source tree; see oracle/ref_shim.py):

    python tests/golden/make_golden.py              # reference_outputs.npz
    python tests/golden/make_golden.py impedance    # impedance_outputs.npz
    python tests/golden/make_golden.py fullsize     # fullsize_outputs.npz (about an hour)

For every case in ``cases.SOLVE_CASES`` the reference solver class is built with
``device='cpu'`` and ``solve(verbose=False, **solve_kwargs)`` is run; tau, D_eff, the iteration
count, the convergence flag and the layer arrays (flux_1d, c_x, tau_x) are stored. For every
case in ``cases.SWEEP_CASES`` the reference loop body (taufactor/taufactor.py:175-182) is run the
given number of times and the padded float32 field is stored bit for bit.

For every case in ``cases.IMPEDANCE_CASES`` the reference's ``ImpedanceSolver`` or
``PeriodicImpedanceSolver`` (taufactor/electrode.py:160-402) is built with ``device='cpu'`` and
solved; its set-up arrays, per-frequency taus, impedances and convergence flags, the summed
iteration count and the final complex128 field go to ``impedance_outputs.npz``.

For every case in ``cases.FULLSIZE_CASES`` (volumes of the benchmark workloads at full size) the
reference solver is run the same way and its iteration count, tau, D_eff and layer flux are
stored, together with the FP64 D_eff of the same operator from ``oracle/fp64.py`` (CG to a
relative residual of 1e-10). For every case in ``cases.DOUBLE_CASES`` the reference is run with
``precision=torch.double`` (float64 sweeps, taufactor.py:24, :33). Both go to
``fullsize_outputs.npz``.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from cases import DOUBLE_CASES, FULLSIZE_CASES, IMPEDANCE_CASES, SOLVE_CASES, SWEEP_CASES  # noqa: E402
from oracle.ref_shim import import_reference  # noqa: E402

CLASS_OF = {
    "binary": "Solver",
    "periodic": "PeriodicSolver",
    "anisotropic": "AnisotropicSolver",
    "multiphase": "MultiPhaseSolver",
    "periodic_multiphase": "PeriodicMultiPhaseSolver",
    "electrode": "ElectrodeSolver",
    "periodic_electrode": "PeriodicElectrodeSolver",
}


def build(tau, kind, img, kw, **extra):
    cls = getattr(tau, CLASS_OF[kind])
    if kind in ("multiphase", "periodic_multiphase"):
        ds = kw.get("diffusivities")
        return cls(img, dict(ds) if ds is not None else None, device="cpu", **extra)
    if kind == "anisotropic":
        return cls(img, kw["spacing"], device="cpu", **extra)
    return cls(img, device="cpu", **extra)


def main():
    import torch

    tau = import_reference()
    if tau is None:
        raise SystemExit("reference source tree not found")
    torch.manual_seed(0)
    out = {}
    for name, (kind, make, kw, solve_kw, _src) in SOLVE_CASES.items():
        img = make()
        with contextlib.redirect_stdout(io.StringIO()):
            s = build(tau, kind, img, kw)
            s.solve(verbose=False, **solve_kw)
        out[f"{name}/tau"] = np.asarray(s.tau, dtype=np.float64)
        out[f"{name}/iter"] = np.asarray(s.iter)
        out[f"{name}/converged"] = np.asarray(bool(s.converged))
        out[f"{name}/c_x"] = np.asarray(s.c_x, dtype=np.float64)
        out[f"{name}/tau_x"] = np.asarray(s.tau_x, dtype=np.float64)
        if kind in ("electrode", "periodic_electrode"):
            out[f"{name}/k_x"] = np.asarray(s.k_x, dtype=np.float64)
            out[f"{name}/k_0"] = np.asarray(s.k_0, dtype=np.float32)
            out[f"{name}/a_x"] = np.asarray(s.a_x, dtype=np.float32)
        else:
            out[f"{name}/D_eff"] = np.asarray(s.D_eff, dtype=np.float64)
            out[f"{name}/flux_1d"] = np.asarray(s.flux_1d, dtype=np.float64)
        print(f"{name:24s} iter={s.iter:5d} tau={np.asarray(s.tau)}")
    for name, (kind, make, kw, n) in SWEEP_CASES.items():
        img = make()
        s = build(tau, kind, img, kw)
        with torch.no_grad():
            for _ in range(n):
                s.apply_boundary_conditions()
                inc = s.sum_weighted_neighbours()
                inc /= s.factor
                inc -= s.field[:, 1:-1, 1:-1, 1:-1]
                inc *= s.cb[s.iter % 2]
                s.field[:, 1:-1, 1:-1, 1:-1] += inc
                s.iter += 1
        out[f"{name}/field"] = s.field.numpy().copy()
        if kind in ("electrode", "periodic_electrode"):
            out[f"{name}/k_0"] = np.asarray(s.k_0, dtype=np.float32)
        print(f"{name:24s} field {tuple(s.field.shape)} after {n} half-sweeps")
    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **out)


def impedance_main():
    tau = import_reference()
    if tau is None:
        raise SystemExit("reference source tree not found")
    out = {}
    for name, (periodic, make, kw, solve_kw, _src) in IMPEDANCE_CASES.items():
        img = make()
        cls = tau.PeriodicImpedanceSolver if periodic else tau.ImpedanceSolver
        with contextlib.redirect_stdout(io.StringIO()):
            s = cls(img, device="cpu", **kw)
            s.solve(verbose=False, **solve_kw)
        out[f"{name}/taus"] = np.array([float(np.asarray(t)[0]) for t in s.taus])
        out[f"{name}/impedance"] = np.array(s.impedance, dtype=np.complex128)
        out[f"{name}/converged_freq"] = np.array(s.converged_freq, dtype=bool)
        out[f"{name}/sum_iter"] = np.asarray(s.sum_iter)
        out[f"{name}/field"] = s.field.numpy()[0].copy()
        out[f"{name}/c_x"] = np.asarray(s.c_x, dtype=np.float64)
        out[f"{name}/vol_x"] = np.asarray(s.vol_x)
        out[f"{name}/a_x"] = np.asarray(s.a_x)
        out[f"{name}/freq_0"] = np.asarray(s.freq_0)
        out[f"{name}/frequency"] = np.asarray(s.frequency)
        out[f"{name}/Z_mean"] = np.asarray(s.Z_mean)
        print(f"{name:18s} sum_iter={s.sum_iter:6d} taus={out[name + '/taus'][:3]}")
    np.savez_compressed(os.path.join(HERE, "impedance_outputs.npz"), **out)


def double_solver(tau, kind):
    """The reference's Solver / PeriodicSolver with float64 sweeps: its public classes do not
    take ``precision`` (taufactor.py:380-385), its base ThroughTransportSolver does (:278-280),
    so this subclass repeats Solver.__init__ with precision=torch.double."""
    import torch

    base = getattr(tau, CLASS_OF[kind])

    class DoubleSolver(base):
        def __init__(self, img, omega=None, D_0=1, device="cuda"):
            self._check_binary_labels(img)
            self.conductive_labels = [1]
            tau.taufactor.ThroughTransportSolver.__init__(self, img, omega=omega, precision=torch.double,
                                                          device=device)
            self.D_0 = D_0
            self.D_mean = np.mean(self.vol_x, axis=1)

    return DoubleSolver


def fullsize_main(only=None):
    import time

    import torch

    from oracle.fp64 import d_eff_fp64
    from oracle.sor import OracleSolve

    tau = import_reference()
    if tau is None:
        raise SystemExit("reference source tree not found")
    torch.set_num_threads(os.cpu_count() or 1)
    path = os.path.join(HERE, "fullsize_outputs.npz")
    out = dict(np.load(path)) if os.path.exists(path) else {}
    for name, (kind, make, kw, solve_kw, _what) in FULLSIZE_CASES.items():
        if only and name not in only:
            continue
        img = make()
        t0 = time.time()
        with contextlib.redirect_stdout(io.StringIO()):
            s = build(tau, kind, img, kw)
            s.solve(verbose=False, **solve_kw)
        t1 = time.time()
        out[f"{name}/iter"] = np.asarray(s.iter)
        out[f"{name}/converged"] = np.asarray(bool(s.converged))
        out[f"{name}/tau"] = np.asarray(s.tau, dtype=np.float64)
        out[f"{name}/D_eff"] = np.asarray(s.D_eff, dtype=np.float64)
        out[f"{name}/flux_1d"] = np.asarray(s.flux_1d, dtype=np.float64)
        del s
        o = OracleSolve(img, kind=kind, diffusivities=kw.get("diffusivities"))
        d64, _, resid = d_eff_fp64(o, rtol=1e-10)
        out[f"{name}/D_eff_fp64"] = np.asarray(d64, dtype=np.float64)
        out[f"{name}/fp64_residual"] = np.asarray(resid, dtype=np.float64)
        print(f"{name:18s} iter={int(out[name + '/iter'])} D_eff={out[name + '/D_eff']} "
              f"fp64={d64} ref {t1 - t0:.0f} s, fp64 {time.time() - t1:.0f} s", flush=True)
        np.savez_compressed(path, **out)
    for name, (kind, make, solve_kw) in DOUBLE_CASES.items():
        if only and name not in only:
            continue
        img = make()
        with contextlib.redirect_stdout(io.StringIO()):
            s = double_solver(tau, kind)(img, device="cpu")
            s.solve(verbose=False, **solve_kw)
        out[f"{name}/iter"] = np.asarray(s.iter)
        out[f"{name}/converged"] = np.asarray(bool(s.converged))
        out[f"{name}/tau"] = np.asarray(s.tau, dtype=np.float64)
        out[f"{name}/D_eff"] = np.asarray(s.D_eff, dtype=np.float64)
        print(f"{name:18s} iter={int(out[name + '/iter'])} D_eff={out[name + '/D_eff']}", flush=True)
        np.savez_compressed(path, **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["impedance"]:
        impedance_main()
    elif sys.argv[1:2] == ["fullsize"]:
        fullsize_main(set(sys.argv[2:]) or None)
    else:
        main()
