"""Drop-in solver classes for TauFactor's through-transport solve on one GB300.

Mirrors the reference's operator surface (tldr-group/taufactor v1.2.1,
taufactor/taufactor.py): the class names, constructor arguments, ``solve()`` arguments and
return value, the attributes it sets (``tau``, ``D_eff``, ``tau_x``, ``c_x``, ``flux_1d``,
``vol_x``, ``D_mean``, ``D_0``, ``iter``, ``converged``, ``walltime``, ``field``), its errors and
warnings, and its convergence rule (layer-flux spread and tau change, checked every 100
half-sweeps). The half-sweeps themselves, the set-up and the layer reductions run as sm_103a
kernels of libtaufactor_gb300 through its C ABI; each half-sweep is the reference's
arithmetic bit for bit.

Deliberate differences:
* a non-CUDA device raises RuntimeError (the reference warns and falls back to the CPU,
  :207-216): there is no CPU path;
* layer means are accumulated in float64 on the device (the reference reduces in float32), so
  ``flux_1d``, ``c_x``, ``tau`` and ``D_eff`` are float64 arrays;
* ``field`` is assembled on access in the reference's padded layout; the solver keeps the
  volume in a z-parity split layout on the device.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings
from timeit import default_timer as timer

import numpy as np
import torch

from . import _capi, autotune
from ._capi import (TF_KIND_ANISOTROPIC, TF_KIND_BINARY, TF_KIND_ELECTRODE, TF_KIND_MULTIPHASE, TF_MAX_PHASES,
                    TF_PERIODIC_Y, TF_PERIODIC_Z, TfGeom, TfOperator, check)
from .percolation import spans_x

F32 = np.float32
INF32 = F32(np.inf)


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def unique_labels(img: np.ndarray) -> np.ndarray:
    """np.unique(img), with a fast path for integer/bool images spanning at most 64 values."""
    a = np.asarray(img)
    if a.size and (a.dtype == bool or a.dtype.kind in "iu"):
        lo, hi = int(a.min()), int(a.max())
        if hi - lo < 64:
            return np.array([v for v in range(lo, hi + 1) if v in (lo, hi) or (a == v).any()], dtype=a.dtype)
    return np.unique(a)


def plane_fraction(mask: np.ndarray) -> np.ndarray:
    """Mean of a bool [B,X,Y,Z] mask over (Y, Z) in float64, [B,X] (taufactor.py:42)."""
    B, X = mask.shape[:2]
    return np.count_nonzero(mask.reshape(B, X, -1), axis=2) / float(np.prod(mask.shape[2:]))


class SORSolver:
    """Template of the red-black SOR solve (taufactor.py:15-269).

    Subclasses define the conductive mask / phase indices and the operator; this class owns
    the device buffers, the half-sweep loop and the convergence checks.
    """

    _kind = TF_KIND_BINARY
    _periodic = 0
    #: set to a list to record (start event, end event, half-sweeps) around every tf_advance call
    event_log = None

    #: hooks of the reference's SORSolver (taufactor.py:70-103) whose arithmetic this package runs
    #: in its own CUDA kernels; a subclass overriding one would be ignored there, so it is refused
    DEVICE_HOOKS = ("return_mask", "init_field", "init_conductive_neighbours", "init_reactive_neighbours",
                    "apply_boundary_conditions", "sum_weighted_neighbours", "vertical_flux")

    def __init__(self, img: np.ndarray, omega: float | None = None, precision=None, device="cuda"):
        self._refuse_overridden_hooks()
        self.cpu_img = self._expand_to_4d(img)
        self.batch_size, self.Nx, self.Ny, self.Nz = self.cpu_img.shape
        # taufactor.py:33: the dtype of the sweeps. Here the sweeps are float32 either way; with
        # torch.float64 every solve ends with a float64 defect correction (refine) and the
        # metrics and `field` are those of the float64 solution.
        if precision not in (None, torch.float32, torch.float64):
            raise ValueError("precision must be None, torch.float32 or torch.float64 "
                             f"(got {precision!r})")
        self.precision = torch.float64 if precision == torch.float64 else torch.float32
        self.device = self._init_device(device)
        if omega is None:
            omega = 2 - math.pi / (1.5 * self.Nx)  # taufactor.py:36-37
        self.omega = omega
        fast = self._device_labels()
        if fast is not None:  # labels uploaded as they are; vol_x from one device pass
            phase, self.vol_x = fast
        else:
            phase, mask = self._phase_indices()
            self.vol_x = plane_fraction(mask)
        self._op = self._operator(float(omega))
        autotune.apply(self, *autotune.default_config(self))
        self._build(phase)
        self.converged = False
        self.old_tau = 0
        self.iter = 0
        self.tau = None
        self.tau_x = None
        self.D_eff = None
        self.walltime = 0.0

    @classmethod
    def _refuse_overridden_hooks(cls):
        own = __name__.split(".")[0]
        for name in cls.DEVICE_HOOKS:
            fn = getattr(cls, name, None)
            if fn is not None and not (getattr(fn, "__module__", None) or "").startswith(own):
                raise NotImplementedError(
                    f"{cls.__name__}.{name} overrides a hook of the reference's SORSolver; taufactor_gb300 "
                    "computes the operator in its own CUDA kernels and cannot call it. Express the operator "
                    "through MultiPhaseSolver (per-label diffusivities), AnisotropicSolver or KappaSolver "
                    "(per-voxel conductivity), or use the reference package for custom hooks.")

    # ------------------------------------------------------------------ hooks
    def _device_labels(self):
        """(phase indices already on the device, vol_x) when the labels can serve as phase
        indices as they are, else None (then _phase_indices runs on the host)."""
        return None

    def _phase_indices(self):
        """uint8 phase indices [B,X,Y,Z] for tf_pack and the bool conductive mask."""
        raise NotImplementedError

    def _operator(self, omega: float) -> TfOperator:
        op = TfOperator()
        op.kind = self._kind
        op.periodic = self._periodic
        op.omega = float(F32(omega))
        op.ghost_lo = 2 * self.top_bc
        op.ghost_hi = 2 * self.bot_bc
        op.ky = op.kz = 1.0
        for i in range(256):
            op.divisor[i] = np.inf
        return op

    # ------------------------------------------------------------------ device state
    def _build(self, phase):
        """phase: uint8 [B,X,Y,Z] numpy array, or a uint8 tensor already on the device."""
        self._lib = _capi.load()
        g = TfGeom()
        check(self._lib.tf_geometry(self.batch_size, self.Nx, self.Ny, self.Nz, self._periodic, C.byref(g)),
              "tf_geometry")
        self._geom = g
        dev = self.device
        with torch.cuda.device(dev):
            self._code = torch.empty(g.code_bytes, dtype=torch.uint8, device=dev)
            self._fa = torch.empty(g.field_elems, dtype=torch.float32, device=dev)
            self._fb = torch.zeros(g.field_elems, dtype=torch.float32, device=dev)
            self._err = torch.zeros(1, dtype=torch.int32, device=dev)
            profile = self._initial_profile().to(dev)
            if isinstance(phase, torch.Tensor):
                phase_dev = phase
            else:
                phase_dev = torch.from_numpy(np.ascontiguousarray(phase, dtype=np.uint8)).to(dev)
            self._phase_dev, self._profile_dev = phase_dev, profile
            self._pack()
            self._flux_dev = torch.empty((self.batch_size, max(self.Nx - 1, 1)), dtype=torch.float64, device=dev)
            self._csum_dev = torch.empty((self.batch_size, self.Nx), dtype=torch.float64, device=dev)
        self._cur, self._other = self._fa, self._fb
        self._field64 = None

    def _initial_profile(self) -> torch.Tensor:
        """float32 [Nx] initial value of a conductive voxel in plane x: the reference's float32
        linspace (taufactor.py:284-286), computed on the host."""
        sh = 1 / (2 * self.Nx)
        return torch.linspace(self.top_bc + sh, self.bot_bc - sh, self.Nx, dtype=torch.float32)

    def _pack(self):
        with torch.cuda.device(self.device):
            check(self._lib.tf_pack(C.byref(self._geom), C.byref(self._op), _ptr(self._phase_dev),
                                    _ptr(self._profile_dev), _ptr(self._code), _ptr(self._fa), self._stream()),
                  "tf_pack")

    def reset(self):
        """Restart the solve from the initial linear field, keeping the device buffers."""
        self._field64 = None
        self._pack()
        self._cur, self._other = self._fa, self._fb
        self.converged = False
        self.old_tau = 0
        self.iter = 0
        self.tau = self.tau_x = self.D_eff = None

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _conductive_table(self):
        t = (C.c_uint8 * 256)()
        if self._kind == TF_KIND_MULTIPHASE:
            for i in range(32):
                t[i] = self._op.conductive[i]
        else:
            t[1] = 1
        return t

    def spans_x_device(self) -> np.ndarray:
        """Whether each volume has a face-connected conductive path from x = 0 to x = Nx-1
        (bool [B]), by the device's union-find labelling (tf_spans_x); the reference labels on
        the host (taufactor.py:318-327, metrics/connectivity.py:138-213)."""
        with torch.cuda.device(self.device):
            labels = torch.empty(self.batch_size * self.Nx * self.Ny * self.Nz, dtype=torch.int32, device=self.device)
            spans = torch.empty(self.batch_size, dtype=torch.int32, device=self.device)
            check(self._lib.tf_spans_x(self.batch_size, self.Nx, self.Ny, self.Nz, _ptr(self._phase_dev),
                                       self._conductive_table(), _ptr(labels), _ptr(spans), _ptr(self._err),
                                       self._stream()), "tf_spans_x")
            out = spans.cpu().numpy() != 0
            err = int(self._err.item())
        if err:
            self._err.zero_()
            raise _capi.TfError(err, "tf_spans_x (device)")
        return out

    def tune(self, half_sweeps: int = 48) -> dict:
        """Pick the fastest tile shape / half-sweeps per launch for these volumes (results unchanged)."""
        return autotune.tune(self, half_sweeps)

    def refine(self, tol: float = 1e-10, max_outer: int = 12, inner_half_sweeps: int | None = None,
               omega: float | None = None, inner: str = "auto"):
        """FP64 defect correction of the current field; returns the relative residual history.

        Keeps the solution in float64, forms r = b - A c in float64 on the device, solves A e = r
        approximately in float32 and adds e in float64, until max over volumes of ||r|| / ||b||
        < tol. The reference has no such step (it iterates in float32 only,
        taufactor.py:172-182). Afterwards the metrics (D_eff, tau, flux_1d, c_x, tau_x) come from
        the float64 field and the float32 field holds its rounding.

        inner: "sor" solves A e = r by inner_half_sweeps float32 sweeps (right-hand side r,
        homogeneous Dirichlet faces; omega: their over-relaxation, default the solve's own;
        2 - 3/Nx needed 9 instead of 13 outer steps on a 256^3 binary volume and 14 instead of 15
        on a 320^3 three-label one). "mg" (binary and multiphase kinds) solves it by conjugate
        gradients preconditioned with a multigrid V-cycle on the same operator, written as
        per-voxel faces (multigrid.KappaMultigrid), to a relative residual of 1e-5; clusters that
        touch neither x face are frozen for it (the anchored system of the FP64 oracle). "auto"
        (the default): "mg" for the binary and multiphase kinds, "sor" for the others.
        """
        if inner not in ("auto", "sor", "mg"):
            raise ValueError('inner must be "auto", "sor" or "mg"')
        if inner == "auto":
            inner = "mg" if self._kind in (TF_KIND_BINARY, TF_KIND_MULTIPHASE) else "sor"
        self.inner_fallback = False  # set when a multigrid inner solve failed and SOR took over
        n_inner = inner_half_sweeps or max(400, 2 * (self.iter or 200))
        solve_e = None
        with torch.cuda.device(self.device):
            if inner == "mg":
                mg = self.multigrid()
                code = self._anchored_code()

                def solve_e(e, r):
                    _, rel_in = mg.solve(e, r, rtol=1e-5, max_iter=max(50, n_inner // 4))
                    ok = bool(np.all(np.isfinite(rel_in)) and rel_in.max() < 0.5)
                    self.inner_fallback = self.inner_fallback or not ok
                    return ok
            else:
                code = self._code if self._kind == TF_KIND_BINARY else self._anchored_code()
            c64, hist = refine_field(self._lib, self._geom, self._op, self._cur, code, self._err,
                                     self._stream(), self.batch_size, tol, max_outer, n_inner, omega, solve_e)
        tau_before = self.tau
        self._field64 = c64
        self.residual_history = hist
        self.tau, _ = self.compute_metrics()
        self.tau = np.where(self.tau == 0, np.inf, self.tau)
        keep_non_percolating(self, tau_before)
        return hist

    def _phase_conductivities(self) -> np.ndarray:
        """float32 conductivity of every phase index of the packed phase map (256 entries)."""
        t = np.zeros(256, dtype=np.float32)
        t[1] = 1.0
        return t

    def multigrid(self):
        """Multigrid preconditioner of refine(inner="mg"): the operator on the anchored phase
        map written as per-voxel faces (kappa = conductivity of the phase index; for the binary
        kind the faces are 1 between conductive neighbours, counted twice on the Dirichlet faces,
        so the factor is the neighbour count of the sweeps)."""
        cached = getattr(self, "_mg", None)
        if cached is not None:
            return cached
        if self._kind not in (TF_KIND_BINARY, TF_KIND_MULTIPHASE):
            raise ValueError("multigrid inner solves need the binary or the multiphase operator")
        from types import SimpleNamespace

        from .multigrid import KappaMultigrid

        g, dev, st = self._geom, self.device, self._stream()
        phase = self._anchored_phase()
        table = torch.from_numpy(self._phase_conductivities()).to(dev)
        kap = table[phase.long()]
        del phase
        f32 = dict(dtype=torch.float32, device=dev)
        ks = torch.empty(g.field_elems, **f32)
        scratch = torch.empty(g.field_elems, **f32)
        check(self._lib.tf_kappa_pack(C.byref(g), C.byref(self._op), _ptr(kap), _ptr(self._profile_dev), _ptr(ks),
                                      _ptr(scratch), st), "tf_kappa_pack")
        del kap, scratch
        plane = g.field_elems // (self.batch_size * self.Nx)
        fx = torch.empty(self.batch_size * (self.Nx + 1) * plane, **f32)
        fy, fz, dv = (torch.empty(g.field_elems, **f32) for _ in range(3))
        check(self._lib.tf_kappa_faces(C.byref(g), _ptr(ks), _ptr(fx), _ptr(fy), _ptr(fz), _ptr(dv), self._periodic,
                                       st), "tf_kappa_faces")
        del ks
        view = SimpleNamespace(device=dev, _op=self._op, batch_size=self.batch_size, Nx=self.Nx, Ny=self.Ny,
                               Nz=self.Nz, _geom=g, _fx=fx, _fy=fy, _fz=fz, _dv=dv)
        self._mg = KappaMultigrid(view)
        return self._mg

    def _anchored_phase(self) -> torch.Tensor:
        """Phase indices (natural layout, uint8) with conductive voxels of clusters that touch
        neither x-face set to 0 (tf_anchored_phase)."""
        cached = getattr(self, "_phase_anchored", None)
        if cached is not None:
            return cached
        n = self.batch_size * self.Nx * self.Ny * self.Nz
        dev = self.device
        labels = torch.empty(n, dtype=torch.int32, device=dev)
        flags = torch.empty(n, dtype=torch.uint8, device=dev)
        phase = torch.empty(n, dtype=torch.uint8, device=dev)
        check(self._lib.tf_anchored_phase(self.batch_size, self.Nx, self.Ny, self.Nz, self._periodic,
                                          _ptr(self._phase_dev), self._conductive_table(), _ptr(labels),
                                          _ptr(flags), _ptr(phase), _ptr(self._err), self._stream()),
              "tf_anchored_phase")
        del labels, flags
        if int(self._err.item()):
            self._err.zero_()
            raise _capi.TfError(_capi.TF_ERR_TIMEOUT, "tf_anchored_phase (device)")
        self._phase_anchored = phase
        return phase

    def _anchored_code(self) -> torch.Tensor:
        """Codes of the system the FP64 refinement solves: conductive voxels of clusters that touch
        neither x-face are frozen (tf_anchored_phase), as in the FP64 oracle. Such a cluster carries
        no flux; under a float32 diagonal (the rounded sum of its faces) its block of the operator
        is nearly singular, so the float32 correction sweeps cannot remove its share of the
        residual and the refinement would stall near 1e-8. The binary kind's integer diagonal
        keeps the block exactly singular, and it uses its own codes."""
        cached = getattr(self, "_code_anchored", None)
        if cached is not None:
            return cached
        phase = self._anchored_phase()
        code = torch.empty_like(self._code)
        scratch = torch.empty(self._geom.field_elems, dtype=torch.float32, device=self.device)
        check(self._lib.tf_pack(C.byref(self._geom), C.byref(self._op), _ptr(phase), _ptr(self._profile_dev),
                                _ptr(code), _ptr(scratch), self._stream()), "tf_pack")
        self._code_anchored = code
        return code

    def _advance(self, n: int):
        """n half-sweeps (reference iterations) starting at colour iter % 2."""
        if n <= 0:
            return
        self._field64 = None
        in_b = C.c_int(0)
        ev = self.event_log
        if ev is not None:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
        with torch.cuda.device(self.device):
            check(self._lib.tf_advance(C.byref(self._geom), C.byref(self._op), _ptr(self._cur), _ptr(self._other),
                                       _ptr(self._code), self.iter % 2, n, _ptr(self._err), C.byref(in_b),
                                       self._stream()), "tf_advance")
        if ev is not None:
            e1.record()
            ev.append((e0, e1, n))
        if in_b.value:
            self._cur, self._other = self._other, self._cur
        self.iter += n

    def _layer_means(self):
        """float64 per-layer means of the x-flux [B,Nx-1] and of the field [B,Nx].

        Taken from the float64 field once refine() has produced one, else from the float32 field.
        """
        with torch.cuda.device(self.device):
            if self._field64 is not None:
                check(self._lib.tf_layer_sums_f64(C.byref(self._geom), C.byref(self._op), _ptr(self._field64),
                                                  _ptr(self._code), _ptr(self._flux_dev), _ptr(self._csum_dev),
                                                  self._stream()), "tf_layer_sums_f64")
                anchored = getattr(self, "_code_anchored", None)
                if anchored is not None:
                    # the flux of the system the refinement solved: clusters that touch neither
                    # x-face carry none (their faces are left out, as in the FP64 oracle); the
                    # field means keep every conductive voxel
                    scratch = torch.empty_like(self._csum_dev)
                    check(self._lib.tf_layer_sums_f64(C.byref(self._geom), C.byref(self._op), _ptr(self._field64),
                                                      _ptr(anchored), _ptr(self._flux_dev), _ptr(scratch),
                                                      self._stream()), "tf_layer_sums_f64")
            else:
                check(self._lib.tf_layer_sums(C.byref(self._geom), C.byref(self._op), _ptr(self._cur),
                                              _ptr(self._code), _ptr(self._flux_dev), _ptr(self._csum_dev),
                                              self._stream()), "tf_layer_sums")
            flux = self._flux_dev.cpu().numpy()
            csum = self._csum_dev.cpu().numpy()
            err = int(self._err.item())
        if err:
            self._err.zero_()
            raise _capi.TfError(err, "tf_advance (device)")
        area = float(self.Ny * self.Nz)
        return flux[:, : self.Nx - 1] / area, csum / area

    @property
    def field(self) -> torch.Tensor:
        """The concentration field in the reference's padded layout [B,Nx+2,Ny+2,Nz+2] (a copy).

        float32; with precision=torch.float64 and a float64 solution present (after refine), the
        float64 field with the same ghost planes."""
        out = torch.empty((self.batch_size, self.Nx + 2, self.Ny + 2, self.Nz + 2), dtype=torch.float32,
                          device=self.device)
        with torch.cuda.device(self.device):
            check(self._lib.tf_unpack(C.byref(self._geom), C.byref(self._op), _ptr(self._cur), _ptr(out),
                                      self._stream()), "tf_unpack")
            if self.precision != torch.float64 or self._field64 is None:
                return out
            nat = torch.empty((self.batch_size, self.Nx, self.Ny, self.Nz), dtype=torch.float64, device=self.device)
            check(self._lib.tf_split_to_natural_f64(C.byref(self._geom), _ptr(self._field64), _ptr(nat),
                                                    self._stream()), "tf_split_to_natural_f64")
            out = out.double()
            out[:, 1:-1, 1:-1, 1:-1] = nat
            if self._periodic:  # ghost copies as the reference's apply_boundary_conditions (:501-505)
                out[:, :, 0, :] = out[:, :, -2, :]
                out[:, :, -1, :] = out[:, :, 1, :]
                out[:, :, :, 0] = out[:, :, :, -2]
                out[:, :, :, -1] = out[:, :, :, 1]
        return out

    @field.setter
    def field(self, value: torch.Tensor):
        shape = (self.batch_size, self.Nx + 2, self.Ny + 2, self.Nz + 2)
        v = torch.as_tensor(value, dtype=torch.float32, device=self.device).reshape(shape).contiguous()
        with torch.cuda.device(self.device):
            check(self._lib.tf_repack(C.byref(self._geom), C.byref(self._op), _ptr(v), _ptr(self._cur),
                                      self._stream()), "tf_repack")

    # ------------------------------------------------------------------ convergence
    def compute_metrics(self):
        raise NotImplementedError

    def plot_stats(self, relative_error):
        """Headless stand-in for the reference's matplotlib plot (taufactor.py:333-352)."""
        i = int(np.argmax(relative_error))
        print(f"Iter: {self.iter}, conv error: {abs(relative_error[i]):.3E}, tau: {self.tau[i]:.5f} "
              f"(batch element {i})")

    def check_convergence(self, verbose, conv_crit, plot_interval):
        """taufactor.py:109-153."""
        self.tau, relative_error = self.compute_metrics()
        if verbose == "per_iter":
            i = int(np.argmax(relative_error))
            print(f"Iter: {self.iter}, conv error: {abs(relative_error[i]):.3E}, tau: {self.tau[i]:.5f} "
                  f"(batch element {i})")
        if verbose == "plot" and self.iter % (100 * plot_interval) == 0:
            self.plot_stats(relative_error)
        if verbose == "debug":
            self.tau_t.append(self.tau)
            if self.iter % (100 * plot_interval) == 0:
                i = int(np.argmax(np.abs(relative_error)))
                print(f"Iter: {self.iter}, conv error: {np.abs(relative_error[i]):.3E}, tau: {self.tau[i]:.5f} "
                      f"(batch element {i})")
        if not np.all(relative_error < conv_crit):
            self.old_tau = self.tau
            return False
        tau_error = np.max(np.abs(self.tau - self.old_tau))
        if not tau_error < 2e-3:
            self.old_tau = self.tau
            return False
        self.tau[self.tau == 0] = np.inf
        return True

    def solve(self, iter_limit=10000, verbose=True, conv_crit=1e-2, plot_interval=10, refine=False):
        """Run half-sweeps until converged or iter_limit (taufactor.py:156-191).

        Half-sweeps between two checks run as fused multi-half-sweep launches with no host
        synchronisation; the check every 100 half-sweeps reads the layer sums back. With
        ``refine=True`` (no reference counterpart) the converged field is then corrected in
        float64 (see refine()) and the returned metrics are those of the refined field.
        """
        if verbose:
            torch.cuda.reset_peak_memory_stats(device=self.device)
        if verbose == "debug":
            self.tau_t = []
        double = self.precision == torch.float64
        if double:
            # float32 sweeps to the reference's rule (flux spreads below ~1e-5 are beyond a
            # float32 field), then the float64 correction
            conv_crit = max(conv_crit, 1e-5)
            if not refine:
                refine = True
        start = timer()
        while not self.converged and self.iter < iter_limit:
            n = min(100 - self.iter % 100, iter_limit - self.iter)
            self._advance(n)
            if self.iter % 100 == 0:
                self.converged = self.check_convergence(verbose, conv_crit, plot_interval)
        if refine:
            hist = self.refine(**(refine if isinstance(refine, dict) else {}))
            if double:
                self.converged = bool(self.converged and hist[-1] < (refine.get("tol", 1e-10)
                                                                      if isinstance(refine, dict) else 1e-10))
        torch.cuda.synchronize(self.device)
        self.walltime = timer() - start
        self._end_simulation(self.iter, verbose)
        if self.tau_x is None:
            return self.tau
        return self.tau_x

    # ------------------------------------------------------------------ helpers
    @staticmethod
    def _expand_to_4d(img) -> np.ndarray:
        """taufactor.py:195-204."""
        if not isinstance(img, np.ndarray):
            raise TypeError("Error: input image must be a NumPy array!")
        if img.ndim == 2:
            img = img[..., None]
        if img.ndim == 3:
            img = img[None, ...]
        if img.ndim != 4:
            raise ValueError("expected [B, X, Y, Z]")
        return img

    @staticmethod
    def _init_device(device) -> torch.device:
        """CUDA only: the reference's CPU fallback (taufactor.py:207-216) becomes an error."""
        dev = torch.device(device)
        if dev.type != "cuda":
            raise RuntimeError(f"taufactor_gb300 runs on CUDA devices only (got device={device!r}); "
                               "use the reference package for CPU solves")
        if not torch.cuda.is_available():
            raise RuntimeError("taufactor_gb300 needs a CUDA device, and none is available")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        return dev

    def _end_simulation(self, iterations: int, verbose):
        """taufactor.py:255-269."""
        if self.converged:
            msg = "converged to"
        else:
            print("Warning: not converged")
            msg = "unconverged value of tau"
        if verbose:
            per = self.walltime / iterations if iterations else 0.0
            print(f"{msg}: {self.tau} after: {iterations} iterations in: {np.around(self.walltime, 4)} s "
                  f"({np.around(per, 4)} s/iter)")
            print(f"GPU-RAM currently {torch.cuda.memory_allocated(device=self.device) / 1e6:.2f} MB "
                  f"(max allocated {torch.cuda.max_memory_allocated(device=self.device) / 1e6:.2f} MB; "
                  f"{torch.cuda.max_memory_reserved(device=self.device) / 1e6:.2f} MB reserved)")


def relative_residual(r2: torch.Tensor, b2: torch.Tensor) -> float:
    """max over volumes of ||r|| / ||b|| from the per-plane float64 sums of r^2 and b^2 ([B, Nx],
    device), reduced on the host: the sums are a few KB, and the host keeps torch's reduction
    kernels (slow to load on first use) out of the solve path."""
    r = r2.cpu().numpy().sum(axis=1)
    b = b2.cpu().numpy().sum(axis=1)
    return float((np.sqrt(r) / np.maximum(np.sqrt(b), 1e-300)).max())


def refine_field(lib, g: TfGeom, op: TfOperator, cur: torch.Tensor, code: torch.Tensor, err: torch.Tensor, stream,
                 batch: int, tol: float, max_outer: int, n_inner: int, omega: float | None = None, solve_e=None):
    """FP64 defect correction of the float32 field `cur` (updated in place with the rounding of
    the result); returns the float64 field and the max-over-volumes relative residual history.
    omega: over-relaxation of the correction sweeps (default: the solve's own). solve_e(e, r):
    another inner solve of A e = r (float32 buffers; may overwrite r) instead of the sweeps; it
    returns False when it made no progress, and the sweeps then take over (that correction is
    dropped and the residual formed again)."""
    gp = C.byref(g)
    op0 = TfOperator.from_buffer_copy(op)
    op0.ghost_lo = op0.ghost_hi = 0.0
    if omega is not None:
        op0.omega = float(F32(omega))
    dev = cur.device
    c64 = torch.empty(g.field_elems, dtype=torch.float64, device=dev)
    check(lib.tf_widen_f64(gp, _ptr(cur), _ptr(c64), stream), "tf_widen_f64")
    rhs = torch.zeros(g.field_elems, dtype=torch.float32, device=dev)
    ea = torch.zeros_like(rhs)
    eb = torch.zeros_like(rhs)
    r2 = torch.empty((batch, g.nx), dtype=torch.float64, device=dev)
    b2 = torch.empty_like(r2)
    hist = []
    for outer in range(max_outer + 1):
        check(lib.tf_residual_f64(gp, C.byref(op), _ptr(c64), _ptr(code), _ptr(rhs), _ptr(r2), _ptr(b2), stream),
              "tf_residual_f64")
        rel = relative_residual(r2, b2)
        hist.append(rel)
        if rel < tol or outer == max_outer:
            break
        if solve_e is not None:
            if solve_e(ea, rhs):
                check(lib.tf_axpy_f64(gp, _ptr(c64), _ptr(ea), stream), "tf_axpy_f64")
            else:
                solve_e = None
            continue
        ea.zero_()
        in_b = C.c_int(0)
        check(lib.tf_advance_rhs(gp, C.byref(op0), _ptr(ea), _ptr(eb), _ptr(code), _ptr(rhs), 0, n_inner, _ptr(err),
                                 C.byref(in_b), stream), "tf_advance_rhs")
        check(lib.tf_axpy_f64(gp, _ptr(c64), _ptr(eb if in_b.value else ea), stream), "tf_axpy_f64")
    check(lib.tf_narrow_f64(gp, C.byref(op), _ptr(c64), _ptr(cur), stream), "tf_narrow_f64")
    return c64, hist


class ThroughTransportSolver(SORSolver):
    """Dirichlet x-faces at (-0.5, 0.5), flux-based metrics (taufactor.py:272-331)."""

    def __init__(self, img, omega=None, precision=None, device="cuda"):
        self.top_bc, self.bot_bc = (-0.5, 0.5)
        super().__init__(img, omega, precision, device)

    def compute_metrics(self):
        """taufactor.py:293-331 on float64 layer means read back from the device."""
        self.flux_1d, c_x = self._layer_means()
        return layer_metrics(self, self.flux_1d, c_x)

    # ------------------------------------------------------------------ operator tensors
    # The reference keeps its operator as tensors (taufactor.py:43-67): the divisor `factor`
    # [B,Nx,Ny,Nz] (inf where a voxel is frozen), the over-relaxation chequerboards `cb` and,
    # for the multiphase solvers, the face diffusivities D_x, D_y, D_z. The kernels here never
    # form them; they are built on first access, on the device, with the reference's formulas.
    @property
    def cb(self):
        """[omega * cb, omega * (1 - cb)] with cb = 1 where (x + y + z) is even (taufactor.py:218-225)."""
        cached = getattr(self, "_cb_tensors", None)
        if cached is None:
            dev = self.device
            par = (torch.arange(self.Nx, device=dev)[:, None, None] + torch.arange(self.Ny, device=dev)[None, :, None]
                   + torch.arange(self.Nz, device=dev)[None, None, :]) % 2
            w = torch.tensor(self.omega, dtype=torch.float64, device=dev)
            zero = torch.zeros((), dtype=torch.float64, device=dev)
            cached = [torch.where(par == 0, w, zero).to(self.precision), torch.where(par == 1, w, zero).to(self.precision)]
            self._cb_tensors = cached
        return cached

    @property
    def factor(self) -> torch.Tensor:
        """The divisor of the update per voxel, [B,Nx,Ny,Nz] (inf = frozen), as the reference's
        init_conductive_neighbours returns it for this solver class."""
        cached = getattr(self, "_factor_tensor", None)
        if cached is None:
            cached = self._build_factor()
            self._factor_tensor = cached
        return cached

    def _labels_tensor(self) -> torch.Tensor:
        return torch.from_numpy(np.ascontiguousarray(self.cpu_img)).to(self.device).to(self.precision)

    def _build_factor(self) -> torch.Tensor:
        raise NotImplementedError(f"{type(self).__name__} has no divisor tensor")



def keep_non_percolating(s, tau_before) -> None:
    """After an FP64 correction: a volume the float32 solve found without a percolating path
    (tau 0, later inf, from an exactly zero layer flux, taufactor.py:318-327) keeps that verdict. In
    float64 its blocked layers carry rounding noise (~1e-17) instead of an exact zero, which the
    reference's zero test would read as a tortuosity of ~1e16."""
    if tau_before is None:
        return
    tb = np.asarray(tau_before, dtype=np.float64)
    dead = np.isinf(tb) | (tb == 0)  # 0 before the convergence check turns it into inf
    if dead.shape != np.shape(s.tau) or not dead.any():
        return
    s.tau = np.where(dead, np.inf, s.tau)
    s.D_eff = np.where(dead, 0.0, s.D_eff)
    if s.tau_x is not None:
        s.tau_x[dead] = 0


def layer_metrics(s, flux_1d: np.ndarray, c_x_raw: np.ndarray):
    """The reference's metric arithmetic on per-layer means (taufactor.py:297-331).

    ``s`` provides Nx, top_bc, bot_bc, D_mean, D_0, vol_x [B,Nx], batch_size, cpu_img and
    conductive_labels; it receives c_x, tau_x and D_eff. Returns (tau, relative_error).
    """
    fl_max = np.max(flux_1d, axis=1)
    fl_min = np.min(flux_1d, axis=1)
    mean_fl = np.mean(flux_1d, axis=1)
    relative_error = np.divide(fl_max - fl_min, fl_max, out=np.full_like(fl_max, np.nan), where=fl_max != 0)
    D_rel = mean_fl * s.Nx / abs(s.top_bc - s.bot_bc)
    tau = np.divide(s.D_mean, D_rel, out=np.full_like(D_rel, np.nan), where=D_rel != 0)
    c_x = np.divide(c_x_raw, s.vol_x, out=np.zeros_like(s.vol_x), where=s.vol_x != 0)
    s.c_x = c_x
    flux_from_c = c_x[:, 1:] - c_x[:, :-1]
    flux_from_c[s.vol_x[:, 1:] == 0] = 0
    flux_from_c[s.vol_x[:, :-1] == 0] = 0
    eps = 0.5 * (s.vol_x[:, :-1] + s.vol_x[:, 1:])
    s.tau_x = np.divide(eps * flux_from_c, flux_1d, out=np.full_like(flux_from_c, np.nan), where=flux_1d != 0)
    spans = None
    for b in range(s.batch_size):
        if (fl_min[b] == 0) or (fl_max[b] == 0) or (mean_fl[b] == 0):
            if hasattr(s, "spans_x_device"):  # the solver's phases are on the device
                if spans is None:
                    spans = s.spans_x_device()
                percolates = bool(spans[b])
            else:
                percolates = spans_x(np.isin(s.cpu_img[b], s.conductive_labels))
            if not percolates:
                print(f"Warning: batch element {b} has no percolating path!")
                relative_error[b] = 0
                D_rel[b] = 0
                tau[b] = 0
                s.tau_x[b, :] = 0
    relative_error[np.isnan(mean_fl)] = 0
    s.D_eff = s.D_0 * D_rel
    return tau, relative_error


class Solver(ThroughTransportSolver):
    """Two-phase solver: 1 = conductive, 0 = not (taufactor.py:355-419)."""

    # a subclass that builds itself through ThroughTransportSolver.__init__ (as the reference's
    # float64 pattern does) has run the reference's host label check itself
    _labels_checked = True

    def __init__(self, img, omega=None, D_0=1, device="cuda"):
        self._labels_checked = not self._labels_go_to_device(img, device)
        if self._labels_checked:
            self._check_binary_labels(img)
        self.conductive_labels = [1]
        super().__init__(img, omega=omega, device=device)
        self.D_0 = D_0
        self.D_mean = np.mean(self.vol_x, axis=1)

    def _check_binary_labels(self, img):
        """taufactor.py:387-397 (same message): every label must be 0 or 1."""
        a = np.asarray(img)
        if a.dtype == bool:
            return
        if a.dtype.kind in "iu":
            ok = a.size > 0 and a.min() >= 0 and a.max() <= 1
        else:
            ok = a.size > 0 and bool(np.logical_or(a == 0, a == 1).all())
        if not ok:
            u = np.unique(img)
            raise ValueError(
                "Input image must only contain 0s and 1s. "
                "Your image must be segmented to use this tool. "
                "If your image has been segmented, ensure your labels are "
                "0 for non-conductive and 1 for conductive phase. "
                f"Your image has the following labels: {u}. "
                "If you have more than one conductive phase, use the multi-phase solver.")

    @staticmethod
    def _labels_go_to_device(img, device) -> bool:
        """uint8 / bool labels on a usable CUDA device are checked there (tf_label_stats) rather
        than by host passes; any other input keeps the reference's host check, which then also
        comes before a device error as in the reference."""
        if not isinstance(img, np.ndarray) or img.dtype not in (np.uint8, np.bool_) or not img.flags.c_contiguous:
            return False
        if img.ndim not in (2, 3, 4) or img.size == 0:
            return False
        try:
            dev = torch.device(device)
        except (RuntimeError, TypeError):
            return False
        planes = img.shape[0] * img.shape[1] if img.ndim == 4 else img.shape[0]
        return dev.type == "cuda" and torch.cuda.is_available() and planes <= 65535

    def _device_labels(self):
        """The labels are the phase indices (1 = conductive): upload them as they are and take the
        0/1 check and the per-plane conductive counts from one pass on the device."""
        if self._labels_checked:
            return None
        lib = _capi.load()
        B, X, Y, Z = self.cpu_img.shape
        with torch.cuda.device(self.device):
            labels = torch.from_numpy(self.cpu_img.view(np.uint8)).to(self.device)
            counts = torch.empty((B, X), dtype=torch.int64, device=self.device)
            top = torch.empty(1, dtype=torch.int32, device=self.device)
            rc = lib.tf_label_stats(B, X, Y, Z, labels.data_ptr(), counts.data_ptr(), top.data_ptr(),
                                    torch.cuda.current_stream(self.device).cuda_stream)
            if rc == _capi.TF_ERR_UNSUPPORTED:
                self._labels_checked = True
                self._check_binary_labels(self.cpu_img)
                return None
            check(rc, "tf_label_stats")
            counts_h = counts.cpu().numpy()
            top_h = int(top.item())
        self._labels_checked = True
        if top_h > 1:
            self._check_binary_labels(self.cpu_img)  # raises the reference's ValueError
        return labels, counts_h / float(Y * Z)

    def _phase_indices(self):
        mask = self.cpu_img == 1
        return mask.astype(np.uint8), mask

    def _operator(self, omega):
        op = super()._operator(omega)
        for n in range(1, 9):
            op.divisor[n] = float(n)
        return op

    def _build_factor(self):
        """Conductive face neighbours, the Dirichlet x-faces counted 2, weighted by (1, Ky, Kz)
        for AnisotropicSolver; y/z wrap for the periodic class (taufactor.py:402-410, :459-471,
        :493-499)."""
        img = self._labels_tensor()
        w = (1.0, getattr(self, "Ky", 1.0), getattr(self, "Kz", 1.0))
        p = torch.nn.functional.pad(img, (1, 1, 1, 1, 1, 1))
        p[:, 0], p[:, -1] = 2, 2
        p[:, :, 0], p[:, :, -1] = 0, 0
        p[:, :, :, 0], p[:, :, :, -1] = 0, 0
        if self._periodic:
            p = p[:, :, 1:-1, 1:-1]
        nn = torch.zeros_like(p)
        for dim in range(1, 4):
            for dr in (1, -1):
                nn += torch.roll(p, dr, dim) * w[dim - 1] if dim > 1 and w[dim - 1] != 1.0 else torch.roll(p, dr, dim)
        nn = nn[:, 1:-1] if self._periodic else nn[:, 1:-1, 1:-1, 1:-1]
        nn[img == 0] = torch.inf
        nn[nn == 0] = torch.inf
        return nn


class PeriodicSolver(Solver):
    """Two-phase solver, periodic in y and z (taufactor.py:481-505)."""

    _periodic = TF_PERIODIC_Y | TF_PERIODIC_Z


def anisotropic_divisors(ky: float, kz: float) -> np.ndarray:
    """float32 diagonal of every neighbour pattern, in the reference's summation order.

    Pattern index 1 + xm + 3 xp + 9 ym + 18 yp + 36 zm + 72 zp (xm, xp in {0,1,2}: 2 = Dirichlet
    face; others in {0,1}); index 0 = non-conductive. AnisotropicSolver.init_conductive_neighbours
    (taufactor.py:459-471) accumulates x-1, x+1, y-1, y+1, z-1, z+1, each times its weight.
    """
    out = np.full(256, np.inf, dtype=F32)
    w = (F32(1.0), F32(1.0), F32(ky), F32(ky), F32(kz), F32(kz))
    for xm in range(3):
        for xp in range(3):
            for ym in range(2):
                for yp in range(2):
                    for zm in range(2):
                        for zp in range(2):
                            s = F32(0)
                            for m, wt in zip((xm, xp, ym, yp, zm, zp), w):
                                s = F32(s + F32(F32(m) * wt))
                            idx = 1 + xm + 3 * xp + 9 * ym + 18 * yp + 36 * zm + 72 * zp
                            out[idx] = s if s != 0 else INF32
    return out


class AnisotropicSolver(Solver):
    """Binary solver with voxel spacing (dx, dy, dz) (taufactor.py:422-478)."""

    _kind = TF_KIND_ANISOTROPIC

    def __init__(self, img, spacing, omega=None, D_0=1, device="cuda:0"):
        if not isinstance(spacing, (list, tuple)) or len(spacing) != 3:
            raise ValueError("spacing must be a list or tuple with three elements (dx, dy, dz)")
        if not all(isinstance(x, (int, float)) for x in spacing):
            raise ValueError("All elements in spacing must be integers or floats")
        if np.max(spacing) / np.min(spacing) > 10:
            warnings.warn("This computation is very questionable for largely different spacings e.g. dz >> dx.")
        dx, dy, dz = spacing
        self.Ky = (dx / dy) ** 2
        self.Kz = (dx / dz) ** 2
        super().__init__(img, omega=omega, D_0=D_0, device=device)

    def _operator(self, omega):
        op = SORSolver._operator(self, omega)
        op.ky = float(F32(self.Ky))
        op.kz = float(F32(self.Kz))
        for i, v in enumerate(anisotropic_divisors(self.Ky, self.Kz)):
            op.divisor[i] = float(v)
        return op


def harmonic_face(a, b) -> F32:
    """float32 2ab/(a+b), 0 if a+b == 0 (taufactor.py:577-583)."""
    a, b = F32(a), F32(b)
    den = F32(a + b)
    if not den > 0:
        return F32(0)
    return F32(F32(F32(F32(2) * a) * b) / den)


class MultiPhaseSolver(ThroughTransportSolver):
    """Per-phase diffusivities with harmonic-mean faces (taufactor.py:508-620)."""

    _kind = TF_KIND_MULTIPHASE

    def __init__(self, img, diffusivities=None, D_scaling=1, omega=None, device="cuda"):
        if diffusivities is None:
            diffusivities = {0: 0, 1: 1}
        if not isinstance(diffusivities, dict):
            raise TypeError("diffusivities must be a dictionary mapping phase labels to diffusivities")
        for phase, D_p in diffusivities.items():
            if not isinstance(phase, (int, np.integer)):
                raise TypeError(f"Phase label must be integer, got {type(phase).__name__}")
            D_p = float(D_p)
            if (not np.isfinite(D_p)) or (D_p < 0):
                raise ValueError(f"Diffusivity for label {phase} must be finite and >= 0, got {D_p}")
        self.Ds = diffusivities
        missing_labels = sorted(int(lbl) for lbl in unique_labels(img) if lbl not in self.Ds)
        if missing_labels:
            warnings.warn("No diffusivity provided for phase label(s) "
                          f"{missing_labels}; assuming these phases are isolating.", UserWarning)
            for lbl in missing_labels:
                self.Ds[lbl] = 0.0
        self.conductive_labels = [lbl for lbl, D_p in self.Ds.items() if D_p > 0]
        super().__init__(img, omega=omega, device=device)
        self.VF = {int(p): np.mean(self.cpu_img == p, axis=(1, 2, 3)) for p in unique_labels(self.cpu_img)}
        self.D_0 = D_scaling
        self.D_mean = np.sum([self.VF[z] * self.Ds.get(z, 0.0) for z in self.VF], axis=0)

    def _phase_indices(self):
        labels = unique_labels(self.cpu_img)
        if len(labels) > TF_MAX_PHASES:
            raise _capi.TfError(_capi.TF_ERR_UNSUPPORTED,
                                f"MultiPhaseSolver with {len(labels)} labels (at most {TF_MAX_PHASES})")
        self._labels = labels
        idx = np.searchsorted(labels, self.cpu_img).astype(np.uint8) + 1
        cond = np.isin(self.cpu_img, np.array(self.conductive_labels, dtype=np.float64)) \
            if self.conductive_labels else np.zeros(self.cpu_img.shape, dtype=bool)
        return idx, cond

    def _phase_conductivities(self) -> np.ndarray:
        """float32 diffusivity of every packed phase index (0 unused, i = label i-1), the values
        of the face table."""
        t = np.zeros(256, dtype=np.float32)
        for a, lbl in enumerate(self._labels, start=1):
            t[a] = F32(self.Ds[int(lbl)] if int(lbl) in self.Ds else self.Ds.get(lbl, 0.0))
        return t

    def _operator(self, omega):
        op = super()._operator(omega)
        labels = self._labels
        op.n_phases = len(labels)
        d = [F32(0)] + [F32(self.Ds[int(lbl)] if int(lbl) in self.Ds else self.Ds.get(lbl, 0.0))
                        for lbl in labels]
        for a in range(32):
            op.conductive[a] = 0
            for b in range(32):
                op.face[a * 32 + b] = 0.0
        for a in range(len(d)):
            op.conductive[a] = 1 if (a > 0 and labels[a - 1] in self.conductive_labels) else 0
            for b in range(len(d)):
                op.face[a * 32 + b] = float(harmonic_face(d[a], d[b]))
        return op


    def _face_tensors(self):
        """(D_x, D_y, D_z): harmonic-mean face diffusivities as the reference builds them
        (taufactor.py:577-596; periodic wrap :626-650), [B,Nx+1,Ny,Nz], [B,Nx,Ny+1,Nz], [B,Nx,Ny,Nz+1]."""
        cached = getattr(self, "_faces_cache", None)
        if cached is not None:
            return cached
        img = self._labels_tensor()
        dmap = torch.zeros_like(img)
        for phase, D_p in self.Ds.items():
            dmap[img == phase] = D_p
        d = torch.nn.functional.pad(dmap, (1, 1, 1, 1, 1, 1))
        d[:, 0] = d[:, 1]
        d[:, -1] = d[:, -2]
        if self._periodic:
            d[:, :, 0, :] = d[:, :, -2, :]
            d[:, :, -1, :] = d[:, :, 1, :]
            d[:, :, :, 0] = d[:, :, :, -2]
            d[:, :, :, -1] = d[:, :, :, 1]

        def hm(a, b):
            den = a + b
            out = torch.zeros_like(den)
            ok = den > 0
            out[ok] = 2 * a[ok] * b[ok] / den[ok]
            return out

        cached = (hm(d[:, :-1, 1:-1, 1:-1], d[:, 1:, 1:-1, 1:-1]), hm(d[:, 1:-1, :-1, 1:-1], d[:, 1:-1, 1:, 1:-1]),
                  hm(d[:, 1:-1, 1:-1, :-1], d[:, 1:-1, 1:-1, 1:]))
        self._faces_cache = cached
        return cached

    @property
    def D_x(self) -> torch.Tensor:
        return self._face_tensors()[0]

    @property
    def D_y(self) -> torch.Tensor:
        return self._face_tensors()[1]

    @property
    def D_z(self) -> torch.Tensor:
        return self._face_tensors()[2]

    def _build_factor(self):
        """Sum of the six faces plus the extra Dirichlet x-face, 0 -> inf (taufactor.py:598-604)."""
        D_x, D_y, D_z = self._face_tensors()
        factor = D_x[:, :-1] + D_x[:, 1:] + D_y[:, :, :-1] + D_y[:, :, 1:] + D_z[:, :, :, :-1] + D_z[:, :, :, 1:]
        factor[:, 0] += D_x[:, 0]
        factor[:, -1] += D_x[:, -1]
        factor[factor == 0] = torch.inf
        return factor

    def phase_gradients(self, conv_crit: float = 1e-3, tol: float = 1e-11, method: str = "mg") -> dict:
        """dD_eff/dD_p for every label p (numpy [B] per label), by the adjoint method.

        Builds the per-voxel field kappa = D[label] (float32, the same faces as this solver,
        bit for bit), solves it to an FP64 relative residual of tol, solves the adjoint and sums
        dD_eff/dkappa over the voxels of each label. method "mg" (default): the FP64 defect
        correction with multigrid inner solves from the initial field (conv_crit is not used);
        "sor": the reference's float32 loop to conv_crit first, then the correction. Only the
        corrected field enters the gradient, so both give it to tol. The derivative is that of
        the operator with float64 faces 2ab/(a+b) (KappaSolver's default): with float32 faces
        D_eff moves in rounding steps. For a label of conductivity 0 the value is not a
        derivative (the label's voxels are outside the system there). No reference counterpart
        (the reference solve runs under no_grad, taufactor.py:172).
        """
        from .kappa import KappaSolver

        labels = self._labels
        img = np.asarray(self.cpu_img)
        B, X, Y, Z = img.shape
        lib = _capi.load()
        on_device = img.dtype == np.uint8
        with torch.cuda.device(self.device):
            st = torch.cuda.current_stream(self.device).cuda_stream
            if on_device:
                # uint8 labels: kappa = D[label] by a 256-entry table and the per-label sums of the
                # gradient on the device (tf_label_map, tf_label_sums)
                table = np.zeros(256, dtype=np.float32)
                slot = np.full(256, -1, dtype=np.int32)
                for i, p in enumerate(labels):
                    table[int(p)] = F32(self.Ds.get(int(p), 0.0))
                    slot[int(p)] = i
                lab = torch.from_numpy(img).to(self.device)
                table_d, slot_d = torch.from_numpy(table).to(self.device), torch.from_numpy(slot).to(self.device)
                kap = torch.empty(img.shape, dtype=torch.float32, device=self.device)
                check(lib.tf_label_map(lab.data_ptr(), lab.numel(), table_d.data_ptr(), kap.data_ptr(), st),
                      "tf_label_map")
            else:
                # other label types: the same table through positions in `labels`, on the host
                idx = np.searchsorted(labels, img)
                lut = np.array([F32(self.Ds.get(int(p), 0.0)) for p in labels], dtype=np.float32)
                kap = torch.from_numpy(np.ascontiguousarray(lut[idx])).to(self.device)
            ks = KappaSolver(kap, periodic=bool(self._periodic), omega=self.omega, D_0=self.D_0, device=self.device)
            ks.solve(conv_crit=conv_crit, refine={"tol": tol}, method=method)
            g = ks.gradient(tol=tol)
            self.kappa_solver = ks
            if on_device:
                part = torch.empty((B * X, len(labels)), dtype=torch.float64, device=self.device)
                check(lib.tf_label_sums(B, X, Y, Z, lab.data_ptr(), g.contiguous().data_ptr(), slot_d.data_ptr(),
                                        len(labels), part.data_ptr(), st), "tf_label_sums")
                sums = part.cpu().numpy().reshape(B, X, len(labels)).sum(axis=1)
            else:
                gh = g.cpu().numpy()
                sums = np.stack([np.bincount(idx[b].ravel(), weights=gh[b].ravel(), minlength=len(labels))
                                 for b in range(B)])
        return {int(p): sums[:, i] for i, p in enumerate(labels)}


class PeriodicMultiPhaseSolver(MultiPhaseSolver):
    """Multiphase, periodic in y and z (taufactor.py:623-656)."""

    _periodic = TF_PERIODIC_Y | TF_PERIODIC_Z


def compute_impedance_batched(R: np.ndarray, C: np.ndarray, freq: np.ndarray) -> np.ndarray:
    """Impedance [B,F] of B transmission lines of Nx RC elements (taufactor/utils.py:75-98):
    from the closed end, Z <- R_k + 1 / (i w C_k + 1 / Z), starting from Z = 1e50."""
    if R.shape != C.shape:
        raise ValueError(f"R and C must have same shape; got {R.shape} vs {C.shape}")
    bs, nx = R.shape
    if freq.ndim == 1:
        w = freq[None, :].repeat(bs, axis=0)
    elif freq.ndim == 2 and freq.shape[0] == bs:
        w = freq
    else:
        raise ValueError("freq must be (F,) or (bs, F)")
    Z = np.full_like(w, 1e50, dtype=complex)
    for k in range(nx - 1, -1, -1):
        Z = R[:, k][:, None] + 1.0 / (1j * w * C[:, k][:, None] + 1.0 / Z)
    return Z


class ElectrodeSolver(SORSolver):
    """Electrode tortuosity (taufactor/electrode.py:13-125): concentration 1 at the inlet x = -1,
    closed outlet, reaction to concentration 0 on every face between the conductive phase and
    the reactive phase. tau = Re Z_sim / Re Z_ideal of the transmission line built from the
    layer fluxes.

    The sweep is the default neighbour sum over the divisor nn + nr * k_0 (nn conductive
    neighbours with the inlet face counted twice, nr reactive neighbours, k_0 per volume as in
    taufactor.py:47-55), computed on the device from the voxel's code.
    """

    _kind = TF_KIND_ELECTRODE

    def __init__(self, img, conductive_label=1, reactive_label=0, omega=None, spacing=None, device="cuda"):
        self.left_bc = 1.0
        self.electrode_bc = 0.0
        self.cond_label = conductive_label
        self.reac_label = reactive_label
        self.dx = spacing or 1
        super().__init__(img, omega=omega, device=device)
        self.vol_x = self._vol_x32
        self.c_x = 0

    def _phase_indices(self):
        """uint8 1 = conductive, 2 = reactive; and the reference's float32 a_x, k_0, vol_x
        (taufactor.py:40-55, electrode.py:36-62), from the same torch float32 operations."""
        if self.batch_size > 256:
            raise ValueError("ElectrodeSolver takes at most 256 volumes per batch")
        cond = self.cpu_img == self.cond_label
        reac = (self.cpu_img == self.reac_label) & ~cond
        mask_t = torch.from_numpy(cond.astype(np.float32))
        vol_x = torch.mean(mask_t, (2, 3))
        r = torch.from_numpy(reac.astype(np.float32))
        if self._periodic:
            rp = torch.nn.functional.pad(r, (0, 0, 0, 0, 1, 1))  # x padded with 0, y/z wrap
            reac_nn = torch.zeros_like(rp)
            for dim in range(1, 4):
                for dr in (1, -1):
                    reac_nn += torch.roll(rp, dr, dim)
            reac_nn = reac_nn[:, 1:-1]
        else:
            rp = torch.nn.functional.pad(r, (1, 1, 1, 1, 1, 1))
            reac_nn = torch.zeros_like(rp)
            for dim in range(1, 4):
                for dr in (1, -1):
                    reac_nn += torch.roll(rp, dr, dim)
            reac_nn = reac_nn[:, 1:-1, 1:-1, 1:-1]
        reac_nn[~torch.from_numpy(cond)] = 0.0
        a_x = torch.sum(reac_nn, (2, 3)) / (self.Ny * self.Nz * self.dx)
        k_0 = torch.mean(vol_x, 1) / torch.mean(a_x * self.dx, 1) / self.Nx ** 2
        self.a_x = a_x.numpy()
        self.k_0 = k_0.numpy()
        self._vol_x32 = vol_x.numpy()
        phase = np.where(cond, 1, np.where(reac, 2, 0)).astype(np.uint8)
        return phase, cond

    def _operator(self, omega):
        op = TfOperator()
        op.kind = self._kind
        op.periodic = self._periodic
        op.omega = float(F32(omega))
        op.ghost_lo = 2 * self.left_bc  # the field's x padding (electrode.py:44)
        op.ghost_hi = 0.0
        op.ky = op.kz = 1.0
        for i in range(256):
            op.divisor[i] = float(self.k_0[i]) if i < len(self.k_0) else np.inf
        return op

    def _initial_profile(self) -> torch.Tensor:
        """electrode.py:38-40: electrode_bc + (left_bc - electrode_bc) cosh(1 - x/Nx) / cosh(1) at
        the voxel centres, in float64, then float32."""
        x = np.arange(self.Nx) + 0.5
        c_init = self.electrode_bc + (self.left_bc - self.electrode_bc) * np.cosh(1 - x / self.Nx) / np.cosh(1)
        return torch.tensor(c_init, dtype=torch.float32)

    def set_k_0(self, k_0):
        """Use these float32 reaction prefactors (one per volume) instead of the ones computed
        from the image. The reference takes k_0 as a float32 torch mean on its host, whose last
        bit depends on the platform's reduction order; this pins a value (e.g. another machine's)."""
        k = np.asarray(k_0, dtype=np.float32).reshape(-1)
        if k.shape[0] != self.batch_size:
            raise ValueError("one k_0 per volume")
        self.k_0 = k
        for b, v in enumerate(k):
            self._op.divisor[b] = float(v)

    def refine(self, tol: float = 1e-10, max_outer: int = 12, inner_half_sweeps: int | None = None,
               omega: float | None = None):
        """FP64 defect correction (SORSolver.refine) of the electrode operator: A c = d c - S(c)
        with d = nn + nr k_0 in the sweep's float32 and the inlet ghost term as b. Its integer
        part keeps clusters cut off from the inlet and from the reactive phase exactly singular, as
        for the binary kind, so the correction uses the solver's own codes. No reference counterpart
        (the reference iterates in float32 only). Afterwards k_x, tau_x and tau come from the
        float64 field."""
        self.c_x = 0
        return super().refine(tol=tol, max_outer=max_outer, inner_half_sweeps=inner_half_sweeps, omega=omega)

    def _anchored_code(self) -> torch.Tensor:
        return self._code

    def _layer_sums_electrode(self):
        with torch.cuda.device(self.device):
            if self._flux_dev.shape[1] != self.Nx:
                self._flux_dev = torch.empty((self.batch_size, self.Nx), dtype=torch.float64, device=self.device)
            if self._field64 is not None:
                check(self._lib.tf_layer_sums_f64(C.byref(self._geom), C.byref(self._op), _ptr(self._field64),
                                                  _ptr(self._code), _ptr(self._flux_dev), _ptr(self._csum_dev),
                                                  self._stream()), "tf_layer_sums_f64")
            else:
                check(self._lib.tf_layer_sums(C.byref(self._geom), C.byref(self._op), _ptr(self._cur),
                                              _ptr(self._code), _ptr(self._flux_dev), _ptr(self._csum_dev),
                                              self._stream()), "tf_layer_sums")
            flux = self._flux_dev.cpu().numpy()
            csum = self._csum_dev.cpu().numpy()
            err = int(self._err.item())
        if err:
            self._err.zero_()
            raise _capi.TfError(err, "tf_advance (device)")
        area = float(self.Ny * self.Nz)
        return flux / area, csum / area

    def compute_metrics(self):
        """electrode.py:64-103 on float64 layer means read back from the device."""
        fluxes, c_raw = self._layer_sums_electrode()
        vol_x = self.vol_x
        c_x = np.divide(c_raw, vol_x, out=np.zeros(c_raw.shape), where=vol_x != 0)
        relative_error = np.max(np.abs(c_x - self.c_x), axis=1)
        self.c_x = c_x
        fluxes_1d = np.concatenate((2 * (self.left_bc - c_x[:, :1]), (-c_x[:, 1:] + c_x[:, :-1])), axis=1)
        fluxes_1d[:, 1:][vol_x[:, 1:] == 0] = 0
        fluxes_1d[:, 1:][vol_x[:, :-1] == 0] = 0
        eps = np.concatenate((vol_x[:, :1], 0.5 * (vol_x[:, :-1] + vol_x[:, 1:])), axis=1)
        self.tau_x = np.divide(eps * fluxes_1d, fluxes, out=np.full_like(fluxes_1d, np.nan), where=fluxes != 0)
        fluxes[:, :-1] -= fluxes[:, 1:]
        self.k_x = np.divide(fluxes, c_x - self.electrode_bc, out=np.zeros_like(c_x),
                             where=(c_x - self.electrode_bc) != 0) / self.k_0[:, None]
        freq = np.mean(eps, axis=1, keepdims=True) / np.mean(self.a_x * self.dx, axis=1, keepdims=True) / self.Nx ** 2 * 2 ** -3
        R = self.tau_x / eps
        R[eps == 0] = 1e30
        R[np.isnan(self.tau_x)] = 1e30
        self.Z_sim = compute_impedance_batched(R, self.a_x * self.dx, freq)
        R_ideal = 1 / np.mean(eps, axis=1)[:, None].repeat(self.Nx, axis=1)
        C_ideal = np.mean(self.a_x * self.dx, axis=1)[:, None].repeat(self.Nx, axis=1)
        self.Z_ideal = compute_impedance_batched(R_ideal, C_ideal, freq)
        tau = self.Z_sim[:, 0].real / self.Z_ideal[:, 0].real
        return tau, relative_error


class PeriodicElectrodeSolver(ElectrodeSolver):
    """Electrode solver, periodic in y and z (electrode.py:128-157)."""

    _periodic = TF_PERIODIC_Y | TF_PERIODIC_Z
