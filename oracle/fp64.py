"""FP64 "truth" for the through-transport solve (test infrastructure only).

Assembles, in scipy.sparse, the same discrete operator that the reference's SOR iteration
converges to (tldr-group/taufactor v1.2.1, taufactor/taufactor.py):

* unknowns: voxels with a finite diagonal (conductive voxels for the binary solvers,
  ``factor < inf`` for the multiphase ones; :402-410, :598-603);
* face conductance 1 between two conductive voxels (binary, :95-103), (dx/dy)^2 and (dx/dz)^2
  on y and z faces (anisotropic, :455-478), the harmonic mean 2ab/(a+b) of the two voxel
  diffusivities (multiphase, :577-596); y and z faces wrap for the periodic solvers (:493-505,
  :626-656);
* Dirichlet inlet/outlet: a voxel on x = 0 (x = Nx-1) couples to the boundary value -0.5
  (+0.5) with twice its boundary-face conductance, because the boundary sits half a voxel away
  (the 2 in the padding of :404 and the extra D_x term of :601-602);
* coefficients exactly as the reference iteration uses them: float32 face values (the float32
  (dx/dy)^2 weights of the anisotropic solver) and, as the diagonal, the reference's float32
  divisor ``factor`` (nn or the float32 sum of faces), so the FP64 solution is the fixed point of
  the reference's own discrete operator.

For the per-voxel conductivity kinds ('kappa', 'periodic_kappa') ``coefficients="f64"`` takes
instead float64 faces 2ab/(a+b) of the float32 kappa values and the exact float64 diagonal: the
smooth operator whose D_eff the product differentiates (its ``KappaSolver`` default).

Voxels of clusters that touch neither Dirichlet face make the operator singular; they carry no
flux at convergence, so they are removed (pinned to 0). The system is solved with
Jacobi-preconditioned CG to a relative residual of 1e-10, and D_eff is formed with the
reference's layer-flux formula (:293-303, :412-419, :615-620) in float64.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components
from scipy.sparse.linalg import cg

from .sor import OracleSolve


def _hm64(a, b):
    """float64 harmonic face 2ab/(a+b), 0 where a + b == 0."""
    s_ = a + b
    return np.where(s_ > 0, 2.0 * a * b / np.where(s_ > 0, s_, 1.0), 0.0)


def _exact(o: OracleSolve, coefficients: str) -> bool:
    if coefficients not in ("f32", "f64"):
        raise ValueError(coefficients)
    if coefficients == "f64" and not hasattr(o, "kappa"):
        raise ValueError('coefficients="f64" applies to the kappa kinds only')
    return coefficients == "f64"


def _face_weights(o: OracleSolve, coefficients: str = "f32"):
    """Conductances of the +x, +y, +z faces of every voxel, [B,X,Y,Z] float64 each.

    The last y/z face wraps to index 0 for periodic solvers and is 0 otherwise; the last x
    face (outlet) is handled as a Dirichlet term, so its entry here is 0.
    """
    B, X, Y, Z = o.batch_size, o.Nx, o.Ny, o.Nz
    if _exact(o, coefficients):
        k = o.kappa.astype(np.float64)
        gx = np.zeros((B, X, Y, Z))
        gx[:, :-1] = _hm64(k[:, :-1], k[:, 1:])
        if o.periodic:
            gy = _hm64(k, np.roll(k, -1, axis=2))
            gz = _hm64(k, np.roll(k, -1, axis=3))
        else:
            gy = np.zeros((B, X, Y, Z))
            gy[:, :, :-1] = _hm64(k[:, :, :-1], k[:, :, 1:])
            gz = np.zeros((B, X, Y, Z))
            gz[:, :, :, :-1] = _hm64(k[:, :, :, :-1], k[:, :, :, 1:])
        return gx, gy, gz, k[:, 0], k[:, -1]
    if o.multiphase:
        gx = np.zeros((B, X, Y, Z))
        gx[:, :-1] = o.D_x[:, 1:-1]
        if o.periodic:
            gy = o.D_y[:, :, 1:].astype(np.float64)
            gz = o.D_z[:, :, :, 1:].astype(np.float64)
        else:
            gy = np.zeros((B, X, Y, Z))
            gy[:, :, :-1] = o.D_y[:, :, 1:-1]
            gz = np.zeros((B, X, Y, Z))
            gz[:, :, :, :-1] = o.D_z[:, :, :, 1:-1]
        gb_lo = o.D_x[:, 0].astype(np.float64)
        gb_hi = o.D_x[:, -1].astype(np.float64)
        return gx, gy, gz, gb_lo, gb_hi
    m = o.mask.astype(np.float64)
    ky = float(np.float32(getattr(o, "Ky", 1.0)))
    kz = float(np.float32(getattr(o, "Kz", 1.0)))
    gx = np.zeros_like(m)
    gx[:, :-1] = m[:, :-1] * m[:, 1:]
    if o.periodic:
        gy = m * np.roll(m, -1, axis=2) * ky
        gz = m * np.roll(m, -1, axis=3) * kz
    else:
        gy = np.zeros_like(m)
        gy[:, :, :-1] = m[:, :, :-1] * m[:, :, 1:] * ky
        gz = np.zeros_like(m)
        gz[:, :, :, :-1] = m[:, :, :, :-1] * m[:, :, :, 1:] * kz
    return gx, gy, gz, m[:, 0], m[:, -1]


def assemble(o: OracleSolve, b: int, coefficients: str = "f32"):
    """Sparse SPD system (A, rhs, index map) of batch element b."""
    X, Y, Z = o.Nx, o.Ny, o.Nz
    gx, gy, gz, gb_lo, gb_hi = (a[b] for a in _face_weights(o, coefficients))
    n = X * Y * Z
    idx = np.arange(n).reshape(X, Y, Z)
    rows, cols, vals = [], [], []
    diag = np.zeros(n)
    for g, nb in ((gx, np.roll(idx, -1, 0)), (gy, np.roll(idx, -1, 1)), (gz, np.roll(idx, -1, 2))):
        sel = g.ravel() > 0
        u = idx.ravel()[sel]
        v = nb.ravel()[sel]
        w = g.ravel()[sel]
        rows += [u, v]
        cols += [v, u]
        vals += [-w, -w]
        np.add.at(diag, u, w)
        np.add.at(diag, v, w)
    rhs = np.zeros(n)
    lo = idx[0].ravel()
    hi = idx[-1].ravel()
    diag[lo] += 2 * gb_lo.ravel()
    rhs[lo] += 2 * gb_lo.ravel() * o.top_bc
    diag[hi] += 2 * gb_hi.ravel()
    rhs[hi] += 2 * gb_hi.ravel() * o.bot_bc
    off = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                        shape=(n, n))
    # keep only clusters that touch a Dirichlet face
    active = diag > 0
    dirichlet = np.zeros(n, dtype=bool)
    dirichlet[lo] |= gb_lo.ravel() > 0
    dirichlet[hi] |= gb_hi.ravel() > 0
    ncomp, comp = connected_components(off, directed=False)
    anchored = np.zeros(ncomp, dtype=bool)
    anchored[comp[dirichlet]] = True
    keep = active & anchored[comp]
    # the reference's float32 divisor (finite where the voxel is updated)
    if not _exact(o, coefficients):
        fac = o.factor[b].astype(np.float64).ravel()
        diag = np.where(np.isfinite(fac) & (diag > 0), fac, diag)
    A = (off + sp.diags(diag)).tocsr()
    k = np.nonzero(keep)[0]
    return A[k][:, k].tocsr(), rhs[k], k


def solve_fp64(o: OracleSolve, rtol: float = 1e-10, maxiter: int = 200000, coefficients: str = "f32"):
    """FP64 field [B,X,Y,Z] (0 outside anchored clusters) and the CG residuals reached."""
    B, X, Y, Z = o.batch_size, o.Nx, o.Ny, o.Nz
    field = np.zeros((B, X, Y, Z))
    resid = np.zeros(B)
    prof = np.linspace(o.top_bc + 0.5 / X, o.bot_bc - 0.5 / X, X)
    for b in range(B):
        A, rhs, k = assemble(o, b, coefficients)
        if len(k) == 0:
            continue
        x0 = np.broadcast_to(prof[:, None, None], (X, Y, Z)).ravel()[k]
        dinv = 1.0 / A.diagonal()
        M = sp.diags(dinv)
        sol, info = cg(A, rhs, x0=x0, rtol=rtol, atol=0.0, maxiter=maxiter, M=M)
        if info != 0:
            raise RuntimeError(f"FP64 CG did not reach rtol={rtol} (info={info})")
        resid[b] = np.linalg.norm(rhs - A @ sol) / max(np.linalg.norm(rhs), 1e-300)
        f = np.zeros(X * Y * Z)
        f[k] = sol
        field[b] = f.reshape(X, Y, Z)
    return field, resid


def layer_flux_fp64(o: OracleSolve, field: np.ndarray, coefficients: str = "f32") -> np.ndarray:
    """Reference layer-flux formula (taufactor.py:412-419, :615-620) in float64, [B,X-1]."""
    d = field[:, 1:] - field[:, :-1]
    if _exact(o, coefficients):
        k = o.kappa.astype(np.float64)
        return (_hm64(k[:, :-1], k[:, 1:]) * d).mean(axis=(2, 3))
    if o.multiphase:
        return (o.D_x[:, 1:-1].astype(np.float64) * d).mean(axis=(2, 3))
    # Solver.vertical_flux zeroes faces whose divisor exceeds 8 (:417-418; for the anisotropic
    # solver this also drops finite divisors above 8)
    ok = o.factor <= 8
    d = d * (ok[:, :-1] & ok[:, 1:])
    return d.mean(axis=(2, 3))


def d_eff_fp64(o: OracleSolve, rtol: float = 1e-10, coefficients: str = "f32"):
    """FP64 D_eff per batch element (D_0 * mean layer flux * Nx / |bc difference|)."""
    field, resid = solve_fp64(o, rtol=rtol, coefficients=coefficients)
    flux = layer_flux_fp64(o, field, coefficients)
    d_rel = flux.mean(axis=1) * o.Nx / abs(o.top_bc - o.bot_bc)
    return o.D_0 * d_rel, field, resid


def adjoint_gradient_fp64(o: OracleSolve, rtol: float = 1e-12, coefficients: str = "f32"):
    """FP64 dD_eff/dkappa [B,X,Y,Z] of a per-voxel conductivity field (kind 'kappa' /
    'periodic_kappa'), by the adjoint method on the operator assembled above.

    J = D_0 * Nx / (|dbc| (Nx-1) Ny Nz) * sum over interior x-faces of g (c[x+1] - c[x]),
    A lam = dJ/dc, dJ/dg_f = explicit - (lam_u - lam_w)(c_u - c_w) for an interior face,
    2 lam_u (bc - c_u) for a Dirichlet face (g = hm(k_u, k_u), dg/dk_u = 1), and
    dg/dk_u = 2 k_w^2 / (k_u + k_w)^2 for g = hm(k_u, k_w). No reference counterpart: the
    reference solve runs under no_grad (taufactor/taufactor.py:172).
    """
    B, X, Y, Z = o.batch_size, o.Nx, o.Ny, o.Nz
    K = o.D_0 * X / (abs(o.top_bc - o.bot_bc) * (X - 1) * Y * Z)
    field, _ = solve_fp64(o, rtol=rtol, coefficients=coefficients)
    grads = np.zeros((B, X, Y, Z))
    exact = _exact(o, coefficients)

    def dface(a, w):
        s_ = a + w
        return np.where(s_ > 0, 2 * w * w / np.where(s_ > 0, s_ * s_, 1.0), 0.0)

    for b in range(B):
        A, _, keep = assemble(o, b, coefficients)
        k64 = o.kappa[b].astype(np.float64)
        # faces between planes x and x+1
        gx = _hm64(k64[:-1], k64[1:]) if exact else o.D_x[b, 1:-1].astype(np.float64)
        dj = np.zeros((X, Y, Z))
        dj[1:] += gx
        dj[:-1] -= gx
        dj *= K
        lam = np.zeros(X * Y * Z)
        if len(keep):
            sol, info = cg(A, dj.ravel()[keep], rtol=rtol, atol=0.0, maxiter=200000,
                           M=sp.diags(1.0 / A.diagonal()))
            if info != 0:
                raise RuntimeError("adjoint CG did not converge")
            lam[keep] = sol
        lam = lam.reshape(X, Y, Z)
        c = field[b]
        k = o.kappa[b].astype(np.float64)
        g = np.zeros((X, Y, Z))
        # x faces: u at x, w at x+1; the explicit term K (c_w - c_u) is the face's flux weight
        du = c[1:] - c[:-1]
        djg = K * du - (lam[:-1] - lam[1:]) * (c[:-1] - c[1:])
        g[:-1] += djg * dface(k[:-1], k[1:])
        g[1:] += djg * dface(k[1:], k[:-1])
        g[0] += 2 * lam[0] * (o.top_bc - c[0])
        g[-1] += 2 * lam[-1] * (o.bot_bc - c[-1])
        for ax in (1, 2):
            if o.periodic:
                cw, lw, kw = np.roll(c, -1, axis=ax), np.roll(lam, -1, axis=ax), np.roll(k, -1, axis=ax)
                djf = -(lam - lw) * (c - cw)
                g += djf * dface(k, kw)
                g += np.roll(djf * dface(kw, k), 1, axis=ax)
            else:
                su = tuple(slice(None, -1) if i == ax else slice(None) for i in range(3))
                sw = tuple(slice(1, None) if i == ax else slice(None) for i in range(3))
                djf = -(lam[su] - lam[sw]) * (c[su] - c[sw])
                g[su] += djf * dface(k[su], k[sw])
                g[sw] += djf * dface(k[sw], k[su])
        grads[b] = g
    return grads


def electrode_fp64(o: OracleSolve, rtol: float = 1e-12):
    """FP64 solution of the ElectrodeSolver operator (electrode.py:13-157, taufactor.py:40-55):
    for conductive voxels d c - (sum of conductive face neighbours) = b, d = the float32 factor
    nn + nr k_0 of the sweeps, b = the inlet ghost value 2 left_bc on x = 0 (the outlet is closed);
    y/z wrap for the periodic kind. Sets o.field to the padded float64 solution and returns
    (tau, k_x) from electrode_metrics on float64 layer means. Voxels of clusters that touch
    neither the inlet nor the reactive phase (singular blocks) keep the values o.field had."""
    B, X, Y, Z = o.batch_size, o.Nx, o.Ny, o.Nz
    field = o.field.astype(np.float64)
    idx = np.arange(X * Y * Z).reshape(X, Y, Z)
    for b in range(B):
        fac = o.factor[b].astype(np.float64)
        cond = (o.mask[b] > 0) & np.isfinite(fac)
        rows, cols = [], []
        for ax in range(3):
            nb = np.roll(idx, -1, ax)
            ok = cond & np.roll(cond, -1, ax)
            if ax == 0 or not o.periodic:  # no wrap across a closed face
                sl = [slice(None)] * 3
                sl[ax] = -1
                ok[tuple(sl)] = False
            u, v = idx[ok], nb[ok]
            rows += [u, v]
            cols += [v, u]
        n = X * Y * Z
        off = sp.csr_matrix((np.ones(sum(len(r) for r in rows)), (np.concatenate(rows), np.concatenate(cols))),
                            shape=(n, n))
        rhs = np.zeros(n)
        rhs[idx[0][cond[0]]] = 2 * o.left_bc
        diag = np.where(cond, fac, 0.0).ravel()
        # keep clusters with an inlet face or a reaction term (non-singular blocks)
        ncomp, comp = connected_components(off, directed=False)
        anchored = np.zeros(ncomp, dtype=bool)
        anchored[comp[idx[0][cond[0]]]] = True
        nn = np.asarray(off.sum(axis=1)).ravel()
        reactive = cond.ravel() & (diag > nn + 2 * (np.arange(n) < Y * Z) * cond.ravel())
        anchored[comp[reactive]] = True
        keep = cond.ravel() & anchored[comp]
        k = np.nonzero(keep)[0]
        A = (sp.diags(diag) - off).tocsr()[k][:, k]
        sol, info = cg(A, rhs[k], rtol=rtol, atol=0.0, maxiter=200000, M=sp.diags(1.0 / A.diagonal()))
        if info != 0:
            raise RuntimeError(f"electrode FP64 CG did not reach rtol={rtol}")
        f = field[b, 1:-1, 1:-1, 1:-1].ravel().copy()
        f[k] = sol
        field[b, 1:-1, 1:-1, 1:-1] = f.reshape(X, Y, Z)
    o.field = field
    o.c_x = 0
    tau, _ = o.electrode_metrics(np.float64)
    return tau, o.k_x
