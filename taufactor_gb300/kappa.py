"""Per-voxel conductivity solve with adjoint gradients (no reference counterpart as an API).

``MultiPhaseSolver`` (taufactor/taufactor.py:508-620) gives every label a diffusivity and couples
voxels by harmonic-mean faces. ``KappaSolver`` takes the diffusivity per voxel directly, a
float32 field kappa >= 0; with kappa = D[label] its faces, factor and half-sweeps equal
``MultiPhaseSolver``'s bit for bit (tests/test_adjoint_gpu.py checks this).

On top of the forward solve (the reference's iteration and convergence rule, plus FP64 defect
correction) it computes dD_eff/dkappa by the adjoint method: the operator is symmetric, so the
adjoint A lam = dD_eff/dc is solved by the same sweeps with a right-hand side, again with FP64
defect correction, and the gradient is assembled per voxel from c and lam on the device. Only
the converged c is kept for the backward pass (``DeffFunction``, a torch.autograd.Function).

The FP64 steps (defect correction, refined D_eff, adjoint) use, by default, float64 faces
2ab/(a+b) of the float32 kappa values with the exact diagonal (``coefficients="f64"``): D_eff is
then a smooth function of kappa and its gradient agrees with finite differences. With float32
faces (``coefficients="f32"``, the reference's operator and what the float32 sweeps use) D_eff
moves in steps of one float32 rounding of a face, which puts about 1e-7/h relative noise into a
central difference of step h. The two refined D_eff differ by about 1e-7 relative.

The FP64 steps solve the anchored system of the FP64 oracle: where kappa has zeros, voxels of
clusters that touch neither x face (no flux passes through them; their block of the operator is
singular) are left out (kappa 0 for the float64 steps; the float32 loop keeps the reference's
operator). The inner solve of each FP64 correction step is either the float32 SOR sweeps
(``inner="sor"``) or conjugate gradients preconditioned by a multigrid V-cycle
(``inner="mg"``, ``multigrid.KappaMultigrid``, the default ``"auto"``).
``solve(method="mg")`` skips the float32 SOR loop and runs the FP64 correction with multigrid
inner solves from the current field (the initial profile or a warm start).

The reference runs its solve under ``torch.no_grad()`` (taufactor.py:172); gradients are pinned
by central finite differences and by an FP64 adjoint on the CPU (``oracle/fp64.py``).
"""
from __future__ import annotations

import ctypes as C
import math
from timeit import default_timer as timer

import numpy as np
import torch

from . import _capi
from ._capi import TF_KIND_MULTIPHASE, TF_PERIODIC_Y, TF_PERIODIC_Z, TfGeom, TfOperator, check
from .solvers import keep_non_percolating, layer_metrics, relative_residual


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class KappaSolver:
    """Through-transport solve on a per-voxel conductivity field.

    kappa     float array [X,Y,Z] or [B,X,Y,Z] (numpy or torch), values >= 0
    periodic  periodic in y and z (as PeriodicMultiPhaseSolver)
    omega     over-relaxation factor (default: the reference's 2 - pi/(1.5 Nx))
    D_0       scaling of D_eff (MultiPhaseSolver's D_scaling)
    coefficients  "f64" (default) or "f32": face conductances of the FP64 steps
    """

    top_bc, bot_bc = -0.5, 0.5

    def __init__(self, kappa, periodic: bool = False, omega=None, D_0=1.0, device="cuda", coefficients="f64"):
        if coefficients not in ("f32", "f64"):
            raise ValueError('coefficients must be "f32" or "f64"')
        self._coeff64 = int(coefficients == "f64")
        self.device = torch.device(device)
        if self.device.type != "cuda" or not torch.cuda.is_available():
            raise RuntimeError("KappaSolver runs on CUDA devices only")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        k = torch.as_tensor(kappa, dtype=torch.float32)
        if k.dim() == 3:
            k = k[None]
        if k.dim() != 4:
            raise ValueError("kappa must be [X,Y,Z] or [B,X,Y,Z]")
        self.batch_size, self.Nx, self.Ny, self.Nz = k.shape
        if self.Nx < 2:
            raise ValueError("need at least two planes along x")
        self.kappa = k.to(self.device).contiguous()
        self.periodic = bool(periodic)
        self.omega = 2 - math.pi / (1.5 * self.Nx) if omega is None else omega
        self.D_0 = D_0
        self._lib = lib = _capi.load()
        # input check, vol_x and D_mean from one device pass (tf_kappa_stats): no torch reductions
        B, X, Y, Z = k.shape
        with torch.cuda.device(self.device):
            pos = torch.empty((B, X), dtype=torch.int64, device=self.device)
            sums = torch.empty((B, X), dtype=torch.float64, device=self.device)
            bad = torch.empty(1, dtype=torch.int32, device=self.device)
            check(lib.tf_kappa_stats(B, X, Y, Z, _ptr(self.kappa), _ptr(pos), _ptr(sums), _ptr(bad), self._stream()),
                  "tf_kappa_stats")
            pos_h, sums_h, bad_h = pos.cpu().numpy(), sums.cpu().numpy(), int(bad.item())
        if bad_h:
            raise ValueError("kappa must be finite and >= 0")
        # every voxel conductive: one cluster touching both x faces, A is nonsingular
        self.all_positive = int(pos_h.sum()) == B * X * Y * Z
        self._mg = None
        self._ks_a = None
        self.inner_fallback = False  # set when a multigrid inner solve failed and SOR took over
        self.vol_x = pos_h / float(Y * Z)
        self.D_mean = sums_h.sum(axis=1) / float(X * Y * Z)
        self.cpu_img = None  # built lazily for the percolation fallback
        self.conductive_labels = [1]
        g = self._geom = TfGeom()
        pflag = (TF_PERIODIC_Y | TF_PERIODIC_Z) if self.periodic else 0
        check(lib.tf_geometry(self.batch_size, self.Nx, self.Ny, self.Nz, pflag, C.byref(g)), "tf_geometry")
        op = self._op = TfOperator()
        op.kind = TF_KIND_MULTIPHASE
        op.periodic = pflag
        op.omega = float(np.float32(self.omega))
        op.ghost_lo, op.ghost_hi = 2 * self.top_bc, 2 * self.bot_bc
        op.ky = op.kz = 1.0
        op.n_phases = 1
        with torch.cuda.device(self.device):
            st = self._stream()
            self._ks = torch.empty(g.field_elems, dtype=torch.float32, device=self.device)
            self._c = torch.empty(g.field_elems, dtype=torch.float32, device=self.device)
            sh = 1 / (2 * self.Nx)
            prof = torch.linspace(self.top_bc + sh, self.bot_bc - sh, self.Nx, dtype=torch.float32).to(self.device)
            check(lib.tf_kappa_pack(C.byref(g), C.byref(op), _ptr(self.kappa), _ptr(prof), _ptr(self._ks),
                                    _ptr(self._c), st), "tf_kappa_pack")
            # the operator's faces and factor, once: the sweeps then divide once per voxel
            plane = g.field_elems // (self.batch_size * self.Nx)
            f32 = dict(dtype=torch.float32, device=self.device)
            self._fx = torch.empty(self.batch_size * (self.Nx + 1) * plane, **f32)
            self._fy = torch.empty(g.field_elems, **f32)
            self._fz = torch.empty(g.field_elems, **f32)
            self._dv = torch.empty(g.field_elems, **f32)
            check(lib.tf_kappa_faces(C.byref(g), _ptr(self._ks), _ptr(self._fx), _ptr(self._fy), _ptr(self._fz),
                                     _ptr(self._dv), pflag, st), "tf_kappa_faces")
            self._flux = torch.empty((self.batch_size, self.Nx - 1), dtype=torch.float64, device=self.device)
            self._csum = torch.empty((self.batch_size, self.Nx), dtype=torch.float64, device=self.device)
        self._c64 = None
        self._f64 = None
        self.iter = 0
        self.converged = False
        self.old_tau = 0
        self.tau = self.D_eff = self.tau_x = None
        self.walltime = 0.0
        self.timings = {}

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    # ---------------------------------------------------------------- forward
    def _advance(self, n: int, field: torch.Tensor, rhs=None, op=None, first_colour=None):
        """n half-sweeps of `field` in place from the packed faces (tf_kappa_advance_faces: one
        half-sweep per launch, HBM-bound; the fused form tf_kappa_advance_fused computes the same
        bits and measured slower on this operator)."""
        check(self._lib.tf_kappa_advance_faces(C.byref(self._geom), C.byref(op or self._op), _ptr(field),
                                               _ptr(self._fx), _ptr(self._fy), _ptr(self._fz), _ptr(self._dv),
                                               _ptr(rhs) if rhs is not None else None,
                                               self.iter % 2 if first_colour is None else first_colour, n,
                                               self._stream()), "tf_kappa_advance_faces")

    def _faces64(self):
        """The float64 faces and diagonal of the FP64 steps (coefficients "f64"), packed once."""
        if self._f64 is None:
            g = self._geom
            plane = g.field_elems // (self.batch_size * self.Nx)
            d = dict(dtype=torch.float64, device=self.device)
            fx = torch.empty(self.batch_size * (self.Nx + 1) * plane, **d)
            fy, fz, dv = (torch.empty(g.field_elems, **d) for _ in range(3))
            check(self._lib.tf_kappa_faces_f64(C.byref(g), _ptr(self._kappa64()), _ptr(fx), _ptr(fy), _ptr(fz),
                                               _ptr(dv), self._stream()), "tf_kappa_faces_f64")
            self._f64 = (fx, fy, fz, dv)
        return self._f64

    def _layer_means(self):
        f, is64 = (self._c64, 1) if self._c64 is not None else (self._c, 0)
        if is64 and self._coeff64:
            check(self._lib.tf_kappa_layer_sums_faces_f64(C.byref(self._geom), _ptr(f), _ptr(self._faces64()[0]),
                                                          _ptr(self._flux), _ptr(self._csum), self._stream()),
                  "tf_kappa_layer_sums_faces_f64")
        else:
            check(self._lib.tf_kappa_layer_sums(C.byref(self._geom), _ptr(f), is64, self._coeff64 & is64,
                                                _ptr(self._kappa64() if is64 else self._ks), _ptr(self._flux),
                                                _ptr(self._csum), self._stream()), "tf_kappa_layer_sums")
        area = float(self.Ny * self.Nz)
        return self._flux.cpu().numpy() / area, self._csum.cpu().numpy() / area

    def compute_metrics(self):
        if self.cpu_img is None:
            self.cpu_img = (self.kappa > 0).to(torch.uint8).cpu().numpy()
        self.flux_1d, c_x = self._layer_means()
        return layer_metrics(self, self.flux_1d, c_x)

    def solve(self, iter_limit=10000, conv_crit=1e-2, verbose=False, refine=False, method="sor"):
        """The reference's loop and convergence rule (taufactor.py:156-191) on this operator
        (method "sor"), then `refine` (False, True or refine()'s keyword arguments). method "mg":
        no float32 loop; the FP64 correction with multigrid inner solves from the current field
        (refine's tol, default 1e-11), converged when its residual reaches tol."""
        if method not in ("sor", "mg"):
            raise ValueError('method must be "sor" or "mg"')
        start = timer()
        if method == "mg":
            opts = dict(refine) if isinstance(refine, dict) else {}
            opts.setdefault("inner", "mg")
            hist = self.refine(**opts)
            self.converged = bool(hist[-1] < opts.get("tol", 1e-11))
            self.walltime = timer() - start
            return self.tau_x
        with torch.cuda.device(self.device):
            while not self.converged and self.iter < iter_limit:
                n = min(100 - self.iter % 100, iter_limit - self.iter)
                self._c64 = None
                self._advance(n, self._c)
                self.iter += n
                if self.iter % 100 == 0:
                    self.tau, rel = self.compute_metrics()
                    if verbose:
                        print(f"Iter: {self.iter}, conv error: {np.max(np.abs(rel)):.3E}")
                    if np.all(rel < conv_crit) and np.max(np.abs(self.tau - self.old_tau)) < 2e-3:
                        self.converged = True
                    else:
                        self.old_tau = self.tau
            if refine:
                self.refine(**(refine if isinstance(refine, dict) else {}))
            torch.cuda.synchronize(self.device)
        self.walltime = timer() - start
        self.tau = np.where(self.tau == 0, np.inf, self.tau)
        return self.tau_x

    def warm_start(self, other: "KappaSolver"):
        """Start from another solver's float32 field (same shape and boundary conditions), zeroed
        where this kappa is 0: perturbed-kappa solves (finite differences, design steps) then
        converge in a few hundred half-sweeps instead of from the linear profile."""
        if (other.batch_size, other.Nx, other.Ny, other.Nz, other.periodic) != \
                (self.batch_size, self.Nx, self.Ny, self.Nz, self.periodic):
            raise ValueError("warm_start needs a solver of the same shape and boundary conditions")
        with torch.cuda.device(self.device):
            torch.where(self._ks > 0, other._c.to(self.device), torch.zeros((), device=self.device), out=self._c)
        self._c64 = None
        self.iter = 0
        self.converged = False
        self.old_tau = 0

    def _inner(self, inner: str) -> str:
        if inner not in ("auto", "sor", "mg"):
            raise ValueError('inner must be "auto", "sor" or "mg"')
        return "mg" if inner == "auto" else inner

    def _kappa64(self) -> torch.Tensor:
        """kappa of the FP64 steps (split layout): the solver's own where kappa > 0 everywhere,
        else with the voxels of clusters that touch neither x face set to 0 (tf_anchored_phase
        on the mask kappa > 0)."""
        if self.all_positive:
            return self._ks
        if self._ks_a is None:
            B, X, Y, Z = self.batch_size, self.Nx, self.Ny, self.Nz
            n = B * X * Y * Z
            dev, st, lib = self.device, self._stream(), self._lib
            mask = (self.kappa > 0).to(torch.uint8)
            labels = torch.empty(n, dtype=torch.int32, device=dev)
            flags = torch.empty(n, dtype=torch.uint8, device=dev)
            keep = torch.empty(n, dtype=torch.uint8, device=dev)
            err = torch.zeros(1, dtype=torch.int32, device=dev)
            table = (C.c_uint8 * 256)()
            table[1] = 1
            pflag = (TF_PERIODIC_Y | TF_PERIODIC_Z) if self.periodic else 0
            check(lib.tf_anchored_phase(B, X, Y, Z, pflag, _ptr(mask), table, _ptr(labels), _ptr(flags), _ptr(keep),
                                        _ptr(err), st), "tf_anchored_phase")
            del labels, flags
            if int(err.item()):
                raise _capi.TfError(_capi.TF_ERR_TIMEOUT, "tf_anchored_phase (device)")
            kap = torch.where(keep.view(B, X, Y, Z) > 0, self.kappa, torch.zeros((), device=dev))
            ks = torch.empty_like(self._ks)
            scratch = torch.empty_like(self._c)
            prof = torch.zeros(self.Nx, dtype=torch.float32, device=dev)
            check(lib.tf_kappa_pack(C.byref(self._geom), C.byref(self._op), _ptr(kap), _ptr(prof), _ptr(ks),
                                    _ptr(scratch), st), "tf_kappa_pack")
            self._ks_a = ks
        return self._ks_a

    def multigrid(self):
        """The multigrid preconditioner of the inner solves (built on first use), on the
        float32 faces of the FP64 steps' kappa."""
        if self._mg is None:
            from types import SimpleNamespace

            from .multigrid import KappaMultigrid

            if self.all_positive:
                view = self
            else:
                g = self._geom
                plane = g.field_elems // (self.batch_size * self.Nx)
                f32 = dict(dtype=torch.float32, device=self.device)
                fx = torch.empty(self.batch_size * (self.Nx + 1) * plane, **f32)
                fy, fz, dv = (torch.empty(g.field_elems, **f32) for _ in range(3))
                check(self._lib.tf_kappa_faces(C.byref(g), _ptr(self._kappa64()), _ptr(fx), _ptr(fy), _ptr(fz),
                                               _ptr(dv), int(self._op.periodic), self._stream()), "tf_kappa_faces")
                view = SimpleNamespace(device=self.device, _op=self._op, batch_size=self.batch_size, Nx=self.Nx,
                                       Ny=self.Ny, Nz=self.Nz, _geom=g, _fx=fx, _fy=fy, _fz=fz, _dv=dv)
            self._mg = KappaMultigrid(view)
        return self._mg

    def _fp64_solve(self, x64, b64, tol, max_outer, n_inner, inner="sor", inner_rtol=1e-5):
        """FP64 defect correction for A x = b (b64 None: the Dirichlet terms); returns history.
        Inner solve of A e = r: n_inner float32 SOR half-sweeps from e = 0, or multigrid
        conjugate gradients to a relative residual of inner_rtol."""
        g, lib, st = self._geom, self._lib, self._stream()
        op0 = TfOperator.from_buffer_copy(self._op)
        op0.ghost_lo = op0.ghost_hi = 0.0
        rhs = torch.zeros(g.field_elems, dtype=torch.float32, device=self.device)
        e = torch.zeros_like(rhs)
        r2 = torch.empty((self.batch_size, self.Nx), dtype=torch.float64, device=self.device)
        b2 = torch.empty_like(r2)
        hist = []
        for outer in range(max_outer + 1):
            if self._coeff64:
                fx, fy, fz, dv = self._faces64()
                check(lib.tf_kappa_residual_faces_f64(C.byref(g), C.byref(self._op), _ptr(x64), _ptr(fx), _ptr(fy),
                                                      _ptr(fz), _ptr(dv), _ptr(b64) if b64 is not None else None,
                                                      _ptr(rhs), _ptr(r2), _ptr(b2), st),
                      "tf_kappa_residual_faces_f64")
            else:
                check(lib.tf_kappa_residual_f64(C.byref(g), C.byref(self._op), _ptr(x64), _ptr(self._kappa64()),
                                                _ptr(b64) if b64 is not None else None, 0, _ptr(rhs), _ptr(r2),
                                                _ptr(b2), st), "tf_kappa_residual_f64")
            rel = relative_residual(r2, b2)
            hist.append(rel)
            if rel < tol or outer == max_outer:
                break
            if inner == "mg":
                _, rel_in = self.multigrid().solve(e, rhs, rtol=inner_rtol, max_iter=max(50, n_inner // 4))
                if not (np.all(np.isfinite(rel_in)) and rel_in.max() < 0.5):
                    # multigrid made no progress on this system: drop this correction and take
                    # the SOR sweeps from here on (the residual is formed again from x64)
                    inner = "sor"
                    self.inner_fallback = True
                    continue
            else:
                e.zero_()
                self._advance(n_inner, e, rhs=rhs, op=op0, first_colour=0)
            check(lib.tf_axpy_f64(C.byref(g), _ptr(x64), _ptr(e), st), "tf_axpy_f64")
        return hist

    def refine(self, tol: float = 1e-11, max_outer: int = 12, inner_half_sweeps=None, inner="auto"):
        """FP64 defect correction of the converged field; metrics from the float64 field.
        inner: "sor" (inner_half_sweeps float32 half-sweeps per step), "mg" (multigrid conjugate
        gradients) or "auto" (multigrid where kappa > 0 everywhere)."""
        t0 = timer()
        inner = self._inner(inner)
        n_inner = inner_half_sweeps or max(400, 2 * (self.iter or 200))
        with torch.cuda.device(self.device):
            g, lib, st = self._geom, self._lib, self._stream()
            c64 = torch.empty(g.field_elems, dtype=torch.float64, device=self.device)
            check(lib.tf_widen_f64(C.byref(g), _ptr(self._c), _ptr(c64), st), "tf_widen_f64")
            self.residual_history = self._fp64_solve(c64, None, tol, max_outer, n_inner, inner)
            check(lib.tf_narrow_f64(C.byref(g), C.byref(self._op), _ptr(c64), _ptr(self._c), st), "tf_narrow_f64")
            self._c64 = c64
            tau_before = self.tau
            self.tau, _ = self.compute_metrics()
            torch.cuda.synchronize(self.device)
        self.tau = np.where(self.tau == 0, np.inf, self.tau)
        keep_non_percolating(self, tau_before)
        self.timings["refine_s"] = timer() - t0
        return self.residual_history

    # ---------------------------------------------------------------- adjoint
    def gradient(self, tol: float = 1e-11, max_outer: int = 12, inner_half_sweeps=None, lam0=None,
                 inner="auto") -> torch.Tensor:
        """dD_eff/dkappa [B,X,Y,Z] (float64, on the device) at the current (refined) solution.

        lam0: optional starting adjoint field (another solver's `lam` of the same shape, e.g. the
        previous step of a design loop); the adjoint field is kept as `lam`. inner: as refine()."""
        inner = self._inner(inner)
        if self._c64 is None:
            self.refine(tol=tol, inner=inner)
        t0 = timer()
        n_inner = inner_half_sweeps or max(400, 2 * (self.iter or 200))
        scale = self.D_0 * self.Nx / (abs(self.bot_bc - self.top_bc) * (self.Nx - 1) * self.Ny * self.Nz)
        with torch.cuda.device(self.device):
            g, lib, st = self._geom, self._lib, self._stream()
            dj = torch.zeros(g.field_elems, dtype=torch.float64, device=self.device)
            check(lib.tf_kappa_adjoint_rhs(C.byref(g), _ptr(self._kappa64()), _ptr(dj), float(scale), self._coeff64,
                                           st), "tf_kappa_adjoint_rhs")
            if lam0 is not None:
                if lam0.numel() != g.field_elems:
                    raise ValueError("lam0 must come from a solver of the same shape")
                lam = lam0.to(device=self.device, dtype=torch.float64).clone()
            else:
                lam = torch.zeros(g.field_elems, dtype=torch.float64, device=self.device)
            self.adjoint_history = self._fp64_solve(lam, dj, tol, max_outer, n_inner, inner)
            self.lam = lam
            grad = torch.empty((self.batch_size, self.Nx, self.Ny, self.Nz), dtype=torch.float64, device=self.device)
            if self._coeff64:
                fx, fy, fz, _ = self._faces64()
                check(lib.tf_kappa_gradient_faces_f64(C.byref(g), C.byref(self._op), _ptr(self._c64), _ptr(lam),
                                                      _ptr(self._kappa64()), _ptr(fx), _ptr(fy), _ptr(fz), _ptr(grad),
                                                      float(scale), float(self.top_bc), float(self.bot_bc), st),
                      "tf_kappa_gradient_faces_f64")
            else:
                check(lib.tf_kappa_gradient(C.byref(g), C.byref(self._op), _ptr(self._c64), _ptr(lam),
                                            _ptr(self._kappa64()), _ptr(grad), float(scale), float(self.top_bc),
                                            float(self.bot_bc), st), "tf_kappa_gradient")
            torch.cuda.synchronize(self.device)
        self.timings["adjoint_s"] = timer() - t0
        return grad

    def field(self) -> torch.Tensor:
        """The float32 field in the reference's padded layout [B,Nx+2,Ny+2,Nz+2]."""
        out = torch.empty((self.batch_size, self.Nx + 2, self.Ny + 2, self.Nz + 2), dtype=torch.float32,
                          device=self.device)
        with torch.cuda.device(self.device):
            check(self._lib.tf_unpack(C.byref(self._geom), C.byref(self._op), _ptr(self._c), _ptr(out),
                                      self._stream()), "tf_unpack")
        return out


class DeffFunction(torch.autograd.Function):
    """D_eff(kappa) as a differentiable torch op: forward = converged, FP64-refined solve;
    backward = adjoint solve. Saves only the solver with its converged field."""

    @staticmethod
    def forward(ctx, kappa: torch.Tensor, periodic: bool = False, conv_crit: float = 1e-3, tol: float = 1e-11,
                method: str = "sor"):
        s = KappaSolver(kappa.detach(), periodic=periodic, device=kappa.device)
        s.solve(conv_crit=conv_crit, refine={"tol": tol}, method=method)
        ctx.solver = s
        ctx.tol = tol
        ctx.squeeze = kappa.dim() == 3
        d = torch.as_tensor(np.asarray(s.D_eff, dtype=np.float64), device=kappa.device)
        return d[0] if ctx.squeeze else d

    @staticmethod
    def backward(ctx, grad_out):
        s = ctx.solver
        g = s.gradient(tol=ctx.tol)
        go = grad_out.reshape(-1, 1, 1, 1).to(g.dtype)
        grad = (g * go).to(torch.float32)
        return (grad[0] if ctx.squeeze else grad), None, None, None, None


def d_eff(kappa: torch.Tensor, periodic: bool = False, conv_crit: float = 1e-3, tol: float = 1e-11,
          method: str = "sor") -> torch.Tensor:
    """Differentiable D_eff of a per-voxel conductivity field (float64 result); method as
    KappaSolver.solve."""
    return DeffFunction.apply(kappa, periodic, conv_crit, tol, method)
