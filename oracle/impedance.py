"""complex128 CPU restatement of TauFactor's impedance (tau_e) solve.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the checker for the CUDA path, never the
thing measured or shipped.

Follows tldr-group/taufactor v1.2.1, ``taufactor/electrode.py``:

* set-up                ``ImpedanceSolver.__init__``                 :167-204
                        (mask, neighbour counts, vol_x, a_x, freq_0, frequencies, Z_mean)
* neighbour counts      ``ImpedanceSolver.count_neighbours``         :235-264
                        ``PeriodicImpedanceSolver.count_neighbours`` :373-396
* initial field         ``ImpedanceSolver.init_field_internal``      :214-233
* frequency loop        ``ImpedanceSolver.solve``                    :266-322
* periodic ghost copy   ``PeriodicImpedanceSolver.apply_boundary_conditions`` :398-402
* input impedance       ``ImpedanceSolver.calc_input_impedance``     :324-330
* metrics               ``ImpedanceSolver.compute_metrics``          :379-392
* convergence           ``SORSolver.check_convergence`` (taufactor/taufactor.py:109-153)
* line impedance        ``compute_impedance`` (taufactor/utils.py:63-72)

The half-sweep keeps the reference's operation order (left-to-right neighbour sum, complex
product (ac - bd, ad + bc), one IEEE rounding per operation). The reference's own complex128
results depend on its platform (vectorised versus scalar loop tails, contraction of the complex
product into fused multiply-adds, reduction order of the means), so parity with it is checked to
a relative tolerance, with identical iteration counts.
"""
from __future__ import annotations

import math

import numpy as np


def compute_impedance(R, C, freq):
    """utils.py:63-72: closed-end RC ladder, Z <- R_i + 1 / (i f C_i + 1 / Z) from the far end."""
    Z = np.full_like(freq, 1e50, dtype=complex)
    for R_i, C_i in zip(R[::-1], C[::-1]):
        Z = R_i + 1.0 / (1j * freq * C_i + 1.0 / Z)
    return Z


def _face_sum(p):
    """Six face neighbours of the interior of a padded [X+2, Y+2, Z+2] array."""
    return (p[2:, 1:-1, 1:-1] + p[:-2, 1:-1, 1:-1] + p[1:-1, 2:, 1:-1] + p[1:-1, :-2, 1:-1]
            + p[1:-1, 1:-1, 2:] + p[1:-1, 1:-1, :-2])


def neighbour_counts(img, cond_label, reac_label, periodic):
    """(mask, nn, nr) of one volume [X, Y, Z] (electrode.py:235-264, :373-396): nn = conductive
    face neighbours with the inlet ghost plane (x = -1) counted 2 and the outlet 0; nr = face
    neighbours with the reactive label (no-flux ghosts, or wrapped in y and z when periodic);
    both 0 outside the conductive phase."""
    mask = (img == cond_label).astype(np.float64)
    reac = (img == reac_label).astype(np.float64)
    if periodic:
        mp = np.pad(mask, ((1, 1), (0, 0), (0, 0)))
        mp[0] = 2.0
        nn = (mp[2:] + mp[:-2] + np.roll(mp, 1, 1)[1:-1] + np.roll(mp, -1, 1)[1:-1]
              + np.roll(mp, 1, 2)[1:-1] + np.roll(mp, -1, 2)[1:-1])
        rp = np.pad(reac, ((1, 1), (0, 0), (0, 0)))
        nr = (rp[2:] + rp[:-2] + np.roll(rp, 1, 1)[1:-1] + np.roll(rp, -1, 1)[1:-1]
              + np.roll(rp, 1, 2)[1:-1] + np.roll(rp, -1, 2)[1:-1])
    else:
        mp = np.pad(mask, 1)
        mp[0, 1:-1, 1:-1] = 2.0
        nn = _face_sum(mp)
        nr = _face_sum(np.pad(reac, 1))
    nn[mask == 0] = 0.0
    nr[mask == 0] = 0.0
    return mask, nn, nr


def setup(img, conductive_label=1, reactive_label=0, spacing=None, mode="tau_e", periodic=False):
    """electrode.py:167-204 for one volume (the reference refuses batches)."""
    img = np.asarray(img)
    if img.ndim == 2:
        img = img[..., None]
    if img.ndim == 4:
        if img.shape[0] != 1:
            raise TypeError("batch_size > 1")
        img = img[0]
    nx, ny, nz = img.shape
    dx = spacing or 1
    mask, nn, nr = neighbour_counts(img, conductive_label, reactive_label, periodic)
    vol_x = mask.sum(axis=(1, 2)) / (ny * nz)
    a_x = nr.sum(axis=(1, 2)) / (ny * nz * dx)
    freq_0 = np.mean(vol_x) / np.mean(a_x * dx) / nx ** 2
    if mode == "tau_e":
        frequency = np.array([freq_0 / 2, freq_0 / 4])
    elif mode == "nyquist":
        frequency = (freq_0 * 2 ** (np.arange(-3, 10, 0.5)))[::-1]
    else:
        raise ValueError(mode)
    Z_mean = compute_impedance(np.full(nx, 1 / np.mean(vol_x)), np.full(nx, np.mean(a_x * dx)), frequency)
    return dict(shape=(nx, ny, nz), mask=mask, nn=nn, nr=nr, vol_x=vol_x, a_x=a_x, dx=dx, freq_0=freq_0,
                frequency=frequency, Z_mean=Z_mean, periodic=periodic)


def init_field(st, frc, left_bc=1.0):
    """electrode.py:214-233: left_bc cosh(l (Nx - x)) / cosh(l Nx) at the voxel centres with
    l = sqrt(i frc mean(a_x[1:-1] dx) / mean(vol_x)), masked, padded (inlet ghost 2 left_bc)."""
    nx, ny, nz = st["shape"]
    x = np.arange(0, nx) + 0.5
    lam = np.sqrt(1j * frc * np.mean(st["a_x"][1:-1] * st["dx"]) / np.mean(st["vol_x"]))
    phi = left_bc * np.cosh(lam * (nx - x)) / np.cosh(lam * nx)
    f = np.zeros((nx + 2, ny + 2, nz + 2), dtype=np.complex128)
    f[1:-1, 1:-1, 1:-1] = st["mask"] * phi[:, None, None]
    f[0, 1:-1, 1:-1] = 2 * left_bc
    return f


def factor_table(frc):
    """1 / (nn + i frc nr) for nn in 0..7, nr in 0..6 by Smith's division (the algorithm of
    torch's and numpy's complex128 reciprocal), 0 where nn + nr = 0; index nn + 8 nr."""
    t = np.zeros(56, dtype=np.complex128)
    for nr in range(7):
        d = nr * frc
        for nn in range(8):
            c = float(nn)
            if nn == 0 and nr == 0:
                continue
            if abs(c) >= abs(d):
                rat = d / c
                scl = 1.0 / (c + d * rat)
                t[nn + 8 * nr] = complex((1.0 + 0.0 * rat) * scl, (0.0 - 1.0 * rat) * scl)
            else:
                rat = c / d
                scl = 1.0 / (d + c * rat)
                t[nn + 8 * nr] = complex((1.0 * rat + 0.0) * scl, (0.0 * rat - 1.0) * scl)
    return t


def periodic_ghosts(f):
    """electrode.py:398-402: y ghosts, then z ghosts, from the opposite interior planes."""
    f[:, 0, :] = f[:, -2, :]
    f[:, -1, :] = f[:, 1, :]
    f[:, :, 0] = f[:, :, -2]
    f[:, :, -1] = f[:, :, 1]


def half_sweep(f, factor, cb, periodic):
    """One pass of the loop body (electrode.py:304-309)."""
    if periodic:
        periodic_ghosts(f)
    inc = _face_sum(f)
    a, b = inc.real, inc.imag
    c, d = factor.real, factor.imag
    inc = (a * c - b * d) + 1j * (a * d + b * c)
    inc = inc - f[1:-1, 1:-1, 1:-1]
    inc = inc.real * cb + 1j * (inc.imag * cb)
    f[1:-1, 1:-1, 1:-1] += inc


def chequerboard(shape, omega):
    a, b, c = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    even = ((a + b + c) % 2 == 0).astype(np.float64)
    return [omega * even, omega * (1 - even)]


def layer_metrics(st, f, c_x, left_bc=1.0):
    """compute_metrics (electrode.py:379-392) with calc_input_impedance (:324-330): returns
    (c_av or None if it holds NaN, relative error, input impedance)."""
    c_av = np.mean(np.abs(f[1:-1, 1:-1, 1:-1]), axis=(1, 2))
    vol_x = st["vol_x"]
    c_av[vol_x > 0] /= vol_x[vol_x > 0]
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = np.array(np.max(np.abs(c_av - c_x)) / (np.max(c_av) - np.min(c_av)))
    if np.any(np.isnan(c_av)):
        return None, rel, None
    first = f[1, 1:-1, 1:-1]
    influx = 2 * left_bc - 2 * first
    influx[first == 0] = 0
    return c_av, rel, left_bc / np.mean(influx)


def solve(st, omega=None, iter_limit=10000, conv_crit=1e-3, left_bc=1.0):
    """electrode.py:266-322 with SORSolver.check_convergence (taufactor.py:109-153)."""
    nx, ny, nz = st["shape"]
    if omega is None:
        omega = 2 - math.pi / (1.5 * nx)
    cb = chequerboard((nx, ny, nz), omega)
    mask, nn, nr = st["mask"], st["nn"], st["nr"]
    code = (nn + 8 * nr).astype(np.int64)
    code[mask == 0] = 0
    Z_ref = st["Z_mean"][-1].real
    f = init_field(st, st["frequency"][0], left_bc)
    c_x = 0
    old_tau = 0
    taus, impedance, converged_freq, iters = [], [], [], []
    sum_iter = 0
    tau = None
    converged = False
    for freq in st["frequency"]:
        frc = freq
        if np.any(np.isnan(f)):
            f = init_field(st, frc, left_bc)
        factor = factor_table(frc)[code]
        impedance.append(0)
        converged = False
        tau = 0
        it = 0
        while not converged and it < iter_limit:
            half_sweep(f, factor, cb[it % 2], st["periodic"])
            it += 1
            if it % 100 == 0:
                c_av, rel, z = layer_metrics(st, f, c_x, left_bc)
                if c_av is None:
                    tau_a, rel_a = np.array([0.0]), np.array([0.0])
                else:
                    c_x = c_av
                    impedance[-1] = z
                    tau_a, rel_a = np.array([z.real / Z_ref]), np.expand_dims(rel, 0)
                tau = tau_a
                if not np.all(rel_a < conv_crit):
                    old_tau = tau
                    continue
                if not np.max(np.abs(tau - old_tau)) < 2e-3:
                    old_tau = tau
                    continue
                tau[tau == 0] = np.inf
                converged = True
        converged_freq.append(converged)
        iters.append(it)
        sum_iter += it
        taus.append(tau)
    return dict(taus=taus, impedance=impedance, converged_freq=converged_freq, sum_iter=sum_iter, iters=iters,
                field=f, c_x=c_x, tau=tau, converged=converged)


def direct_field(st, frc, left_bc=1.0):
    """The fixed point of the half-sweeps at one frequency, by a sparse direct solve: on every
    voxel with a non-zero factor, (nn + i frc nr) c - sum of its face neighbours = the inlet
    ghost's 2 left_bc; c = 0 elsewhere. Padded complex128 [X+2, Y+2, Z+2] like the solver's."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    nx, ny, nz = st["shape"]
    nn, nr, mask = st["nn"], st["nr"], st["mask"]
    live = (mask != 0) & ((nn + nr) != 0)
    idx = -np.ones((nx, ny, nz), dtype=np.int64)
    idx[live] = np.arange(int(live.sum()))
    rows, cols, vals = [], [], []
    rhs = np.zeros(int(live.sum()), dtype=np.complex128)
    per = st["periodic"]
    for x, y, z in zip(*np.nonzero(live)):
        i = idx[x, y, z]
        rows.append(i)
        cols.append(i)
        vals.append(nn[x, y, z] + 1j * frc * nr[x, y, z])
        for dx, dy, dz in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
            u, v, w = x + dx, y + dy, z + dz
            if u < 0:
                rhs[i] += 2 * left_bc
                continue
            if u >= nx:
                continue
            if per:
                v, w = v % ny, w % nz
            elif not (0 <= v < ny and 0 <= w < nz):
                continue
            j = idx[u, v, w]
            if j >= 0:
                rows.append(i)
                cols.append(j)
                vals.append(-1.0)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(len(rhs), len(rhs)))
    c = spla.spsolve(A.tocsc(), rhs)
    f = np.zeros((nx + 2, ny + 2, nz + 2), dtype=np.complex128)
    f[1:-1, 1:-1, 1:-1][live] = c
    f[0, 1:-1, 1:-1] = 2 * left_bc
    return f


def input_impedance(f, left_bc=1.0):
    """calc_input_impedance (electrode.py:324-330) of a padded field."""
    first = f[1, 1:-1, 1:-1]
    influx = 2 * left_bc - 2 * first
    influx[first == 0] = 0
    return left_bc / np.mean(influx)
