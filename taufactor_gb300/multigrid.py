"""Multigrid-preconditioned conjugate gradients for the float32 correction solve A e = r of the
per-voxel conductivity operator (KappaSolver's FP64 defect correction).

No reference counterpart: the reference solves only by red-black SOR (taufactor.py:156-191), and
so does the float32 solve to its conv_crit here. Inside the FP64 defect correction any convergent
inner method may stand in for the SOR sweeps, since the float64 residual decides when the field
is done. SOR needs O(nx) sweeps per decade of residual; a V-cycle reduces every error scale at
once, so the inner solve costs a few dozen V-cycles at any size.

Levels: the solver's own geometry and packed float32 faces, then coarse levels that halve every
axis of extent >= 4 (tf_mg_coarsen: aggregates of 2 cells per halved axis, faces summed over the
coarse interface and scaled by 1/2 along a halved normal axis) until no extent can be halved; a
periodic axis is halved only while its half stays even (an odd periodic extent couples cells of
one colour across the wrap).
Smoother: tf_kappa_advance_faces with omega 1 (red-black Gauss-Seidel), `smooth` red/black pairs
before the coarse correction and the same number in the reverse colour order after it, so the
V-cycle is a symmetric positive-definite preconditioner; the coarsest level takes an odd number
of half-sweeps (a palindrome). Two pairs (the default) took the fewest milliseconds per solve
to 1e-5 on a 320^3 kappa field (5 iterations, against 13 with one pair) and on 4 x 256^3
blurred porous volumes (19 against 34; three pairs: 15 iterations, about as fast). Conjugate
gradients run in float32 with float64-accumulated dot products in a fixed order and per-volume
step lengths (tf_mg_dot, tf_pcg_update_*).

Use it for operators whose every cluster touches a Dirichlet face (kappa > 0 everywhere is the
usual case); a cluster cut off from both x faces makes A singular there.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _capi
from ._capi import TfGeom, TfOperator, check


def _ptr(t):
    return t.data_ptr() if t is not None else None


class _Level:
    def __init__(self, geom, dims, fx, fy, fz, dv, e, b):
        self.geom, self.dims = geom, dims
        self.fx, self.fy, self.fz, self.dv = fx, fy, fz, dv
        self.e, self.b = e, b


def level_dims(dims, periodic: int, max_levels: int = 40) -> list:
    """Extents (nx, ny, nz) of every level, finest first: each coarser level halves every extent
    >= 4 (rounding up), a periodic one (TF_PERIODIC_Y / _Z bits of `periodic`) only while the
    half stays even, until no extent can be halved."""
    per = (False, bool(periodic & 1), bool(periodic & 2))
    out = [tuple(int(d) for d in dims)]
    while len(out) < max_levels:
        cd = tuple((d + 1) // 2 if d >= 4 and (not p or d % 4 == 0) else d for d, p in zip(out[-1], per))
        if cd == out[-1]:
            break
        out.append(cd)
    return out


class KappaMultigrid:
    """V-cycle PCG on a KappaSolver's operator (float32 faces, homogeneous Dirichlet x faces).

    solver      a KappaSolver (its geometry, periodicity and packed faces)
    smooth      red/black Gauss-Seidel pairs before and after each coarse correction
    scale       coarse face factor along a halved normal axis (1/2: re-discretisation)
    omega       over-relaxation of the smoothing half-sweeps (any value in (0, 2) keeps the
                palindromic V-cycle symmetric)
    """

    def __init__(self, solver, smooth: int = 2, scale: float = 0.5, omega: float = 1.0):
        if smooth < 1:
            raise ValueError("smooth must be >= 1")
        if not 0.0 < omega < 2.0:
            raise ValueError("omega must lie in (0, 2)")
        self._lib = lib = _capi.load()
        self.device = solver.device
        self.smooth = int(smooth)
        self.periodic = int(solver._op.periodic)
        op = self._op = TfOperator.from_buffer_copy(solver._op)
        op.omega = float(np.float32(omega))
        op.ghost_lo = op.ghost_hi = 0.0
        B = solver.batch_size
        self.batch = B
        dims = (solver.Nx, solver.Ny, solver.Nz)
        f32 = dict(dtype=torch.float32, device=self.device)
        g0 = solver._geom
        with torch.cuda.device(self.device):
            st = torch.cuda.current_stream(self.device).cuda_stream
            self.levels = [_Level(g0, dims, solver._fx, solver._fy, solver._fz, solver._dv, None, None)]
            # a periodic extent is halved only while the half stays even, so every periodic level
            # keeps a proper red/black colouring across the wrap
            for cd in level_dims(dims, self.periodic)[1:]:
                g = TfGeom()
                check(lib.tf_geometry(B, cd[0], cd[1], cd[2], self.periodic, C.byref(g)), "tf_geometry")
                plane = g.field_elems // (B * cd[0])
                fx = torch.empty(B * (cd[0] + 1) * plane, **f32)
                fy, fz, dv = (torch.empty(g.field_elems, **f32) for _ in range(3))
                prev = self.levels[-1]
                check(lib.tf_mg_coarsen(C.byref(prev.geom), _ptr(prev.fx), _ptr(prev.fy), _ptr(prev.fz), C.byref(g),
                                        _ptr(fx), _ptr(fy), _ptr(fz), _ptr(dv), self.periodic, float(scale), st),
                      "tf_mg_coarsen")
                self.levels.append(_Level(g, cd, fx, fy, fz, dv, torch.zeros(g.field_elems, **f32),
                                          torch.zeros(g.field_elems, **f32)))
            # odd length: a palindrome of half-sweeps from zero, so the coarsest solve is symmetric
            self.coarse_half_sweeps = 2 * sum(self.levels[-1].dims) + 1
            n = g0.field_elems
            self.levels[0].e = torch.zeros(n, **f32)  # z = M^-1 r of the conjugate gradients
            self._p = torch.zeros(n, **f32)
            self._q = torch.zeros(n, **f32)
            self._part = torch.empty(2 * B * solver.Nx * solver.Ny, dtype=torch.float64, device=self.device)
            self._d = [torch.empty(2 * B, dtype=torch.float64, device=self.device) for _ in range(3)]
        self.history = []

    def _st(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _smooth(self, L, b, first_colour, n):
        """n half-sweeps of L.e in place with right-hand side b (tf_kappa_advance_faces; the fused
        form computes the same bits and measured slower on this operator)."""
        check(self._lib.tf_kappa_advance_faces(C.byref(L.geom), C.byref(self._op), _ptr(L.e), _ptr(L.fx),
                                               _ptr(L.fy), _ptr(L.fz), _ptr(L.dv), _ptr(b), first_colour, n,
                                               self._st()), "tf_kappa_advance_faces")

    def vcycle(self, level: int, b: torch.Tensor) -> torch.Tensor:
        """The V-cycle from zero applied to b on `level`; returns the buffer holding the result
        (the level's e)."""
        L = self.levels[level]
        L.e.zero_()
        if level == len(self.levels) - 1:
            self._smooth(L, b, 0, self.coarse_half_sweeps)
            return L.e
        self._smooth(L, b, 0, 2 * self.smooth)
        Cl = self.levels[level + 1]
        lib, st = self._lib, self._st()
        check(lib.tf_mg_restrict(C.byref(L.geom), _ptr(L.e), _ptr(b), _ptr(L.fx), _ptr(L.fy), _ptr(L.fz), _ptr(L.dv),
                                 C.byref(Cl.geom), _ptr(Cl.b), st), "tf_mg_restrict")
        ec = self.vcycle(level + 1, Cl.b)
        check(lib.tf_mg_prolong(C.byref(Cl.geom), _ptr(ec), C.byref(L.geom), _ptr(L.e), self.periodic, st),
              "tf_mg_prolong")
        self._smooth(L, b, 1, 2 * self.smooth)
        return L.e

    def _dot(self, out, a1, b1, a2=None, b2=None):
        check(self._lib.tf_mg_dot(C.byref(self.levels[0].geom), _ptr(a1), _ptr(b1), _ptr(a2), _ptr(b2),
                                  _ptr(self._part), _ptr(out), self._st()), "tf_mg_dot")

    def solve(self, x: torch.Tensor, r: torch.Tensor, rtol: float = 1e-5, max_iter: int = 200):
        """Approximately solve A x = r (float32 split-layout buffers of the fine level): x is
        overwritten with the solution, r with the final residual. Stops when every volume's
        residual norm is below rtol times its initial one. Returns (iterations, relative norms)."""
        lib, L0 = self._lib, self.levels[0]
        g = C.byref(L0.geom)
        B = self.batch
        p, q = self._p, self._q
        rz, rz_new, rr = self._d
        with torch.cuda.device(self.device):
            st = self._st()
            x.zero_()
            z = self.vcycle(0, r)
            p.copy_(z)
            self._dot(rz, r, z, r, r)
            rr0 = rz[B:].cpu().numpy().copy()
            rr0[rr0 <= 0] = 1.0
            rel = np.sqrt(np.maximum(rz[B:].cpu().numpy(), 0.0) / rr0)
            it = 0
            while it < max_iter and rel.max() >= rtol:
                it += 1
                check(lib.tf_mg_apply(g, _ptr(p), _ptr(L0.fx), _ptr(L0.fy), _ptr(L0.fz), _ptr(L0.dv), _ptr(q), st),
                      "tf_mg_apply")
                self._dot(rr, p, q)  # rr[:B] = p.q
                check(lib.tf_pcg_update_xr(g, _ptr(x), _ptr(r), _ptr(p), _ptr(q), _ptr(rz), _ptr(rr), st),
                      "tf_pcg_update_xr")
                z = self.vcycle(0, r)
                self._dot(rz_new, r, z, r, r)
                rel = np.sqrt(np.maximum(rz_new[B:].cpu().numpy(), 0.0) / rr0)
                check(lib.tf_pcg_update_p(g, _ptr(p), _ptr(z), _ptr(rz_new), _ptr(rz), st), "tf_pcg_update_p")
                rz, rz_new = rz_new, rz
            self._d = [rz, rz_new, rr]
        self.history.append((it, float(rel.max())))
        return it, rel
