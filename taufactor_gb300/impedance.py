"""Impedance (tau_e) solvers on one GB300: ``ImpedanceSolver`` and ``PeriodicImpedanceSolver``.

Drop-in for taufactor/electrode.py:160-402 (tldr-group/taufactor v1.2.1): the same constructor
arguments, ``solve()`` arguments and printed output, the attributes it sets (``mask``,
``cond_nn``, ``reac_nn``, ``vol_x``, ``a_x``, ``freq_0``, ``frequency``, ``Z_mean``, ``field``,
``impedance``, ``taus``, ``converged_freq``, ``sum_iter``, ``c_x``, ``tau``, ``iter``,
``converged``, ``walltime``) and the reference's frequency loop: the frequencies are solved in
order, each from the previous one's field (re-initialised only if it holds a NaN), each until
the convergence rule of taufactor.py:109-153 holds on the layer means of |c| checked every 100
half-sweeps, or iter_limit.

The complex128 field lives on the device in the reference's padded layout, so ``field`` is the
solver's own tensor. Set-up (neighbour codes, plane counts), the half-sweeps, the periodic ghost
copies and the per-plane reductions run as sm_103a kernels of libtaufactor_gb300
(``tf_impedance_*``); the host keeps the reference's scalar arithmetic (frequencies, the ideal
line impedance Z_mean, the analytic initial profile, the 56-entry factor table, the metrics on
the [Nx] layer means).

``solve_frequencies()`` (no reference counterpart) solves all frequencies side by side as
independent systems, each from its own analytic profile, in one set of launches.

Deliberate differences: a non-CUDA device raises RuntimeError; ``plot_stats`` prints instead of
plotting.
"""
from __future__ import annotations

import ctypes as C
import math
from timeit import default_timer as timer

import numpy as np
import torch

from . import _capi
from ._capi import TF_IMP_TABLE, check
from .solvers import SORSolver


def compute_impedance(R, C_, freq):
    """Impedance of a closed-end RC ladder (taufactor/utils.py:63-72): from the last element,
    Z <- R_i + 1 / (i f C_i + 1 / Z), starting from Z = 1e50."""
    Z = np.full_like(freq, 1e50, dtype=complex)
    for R_i, C_i in zip(R[::-1], C_[::-1]):
        Z = R_i + 1.0 / (1j * freq * C_i + 1.0 / Z)
    return Z


def factor_table(frc: float) -> np.ndarray:
    """complex128 [56]: 1 / (nn + i frc nr) at index nn + 8 nr (nn 0..7, nr 0..6), 0 where
    nn + nr = 0 (electrode.py:297-300). Smith's division, the algorithm of the reference's torch
    complex reciprocal, in Python floats (one rounding per operation on every host)."""
    t = np.zeros(TF_IMP_TABLE, dtype=np.complex128)
    frc = float(frc)
    for nr in range(7):
        d = nr * frc
        for nn in range(8):
            if nn == 0 and nr == 0:
                continue
            c = float(nn)
            if abs(c) >= abs(d):
                rat = d / c
                scl = 1.0 / (c + d * rat)
                t[nn + 8 * nr] = complex((1.0 + 0.0 * rat) * scl, (0.0 - 1.0 * rat) * scl)
            else:
                rat = c / d
                scl = 1.0 / (d + c * rat)
                t[nn + 8 * nr] = complex((1.0 * rat + 0.0) * scl, (0.0 * rat - 1.0) * scl)
    return t


class ImpedanceSolver(SORSolver):
    """Electrode tortuosity from the complex impedance of the pore network (electrode.py:160-366):
    potential 1 at the inlet x = -1, closed outlet, a capacitive sink i frc on every face between
    the conductive and the reactive phase; tau = Re Z_sim / Re Z_mean at the last frequency."""

    _periodic = 0

    def __init__(self, img, conductive_label=1, reactive_label=0, omega=None, spacing=None, mode="tau_e",
                 device="cuda"):
        self.left_bc = 1.0
        self.electrode_bc = 0.0
        self.cond_label = conductive_label
        self.reac_label = reactive_label
        self.dx = spacing or 1
        # SORSolver.__init__ (taufactor.py:24-69) with precision=torch.double
        self.cpu_img = self._expand_to_4d(img)
        self.batch_size, self.Nx, self.Ny, self.Nz = self.cpu_img.shape
        self.device = self._init_device(device)
        self.precision = torch.double
        if omega is None:
            omega = 2 - math.pi / (1.5 * self.Nx)
        self.omega = omega
        self.field = None
        self.factor = None
        self.converged = False
        self.old_tau = 0
        self.iter = 0
        self.tau = None
        self.tau_x = None
        self.D_eff = None
        self.walltime = 0.0
        if self.batch_size > 1:
            raise TypeError("Error: The ImpedanceSolver is only implemented for batch_size=1! "
                            "TODO: vectorize impedance solver for batching.")
        self._lib = _capi.load()
        img0 = self.cpu_img[0]
        phase = ((img0 == self.cond_label).astype(np.uint8) | ((img0 == self.reac_label).astype(np.uint8) << 1))
        dev = self.device
        with torch.cuda.device(dev):
            phase_dev = torch.from_numpy(np.ascontiguousarray(phase)).to(dev)
            self._code = torch.empty((self.Nx, self.Ny, self.Nz), dtype=torch.uint8, device=dev)
            counts = torch.empty((self.Nx, 2), dtype=torch.int64, device=dev)
            check(self._lib.tf_impedance_pack(self.Nx, self.Ny, self.Nz, self._periodic, phase_dev.data_ptr(),
                                              self._code.data_ptr(), counts.data_ptr(), self._stream()),
                  "tf_impedance_pack")
            counts = counts.cpu().numpy()
            self._abs = torch.empty((1, self.Nx), dtype=torch.float64, device=dev)
            self._influx = torch.empty(2, dtype=torch.float64, device=dev)
            self._nan = torch.zeros(1, dtype=torch.int32, device=dev)
            self._table = torch.zeros(TF_IMP_TABLE, dtype=torch.complex128, device=dev)
        # electrode.py:186-187 (integer sums, exact in float64)
        self.vol_x = counts[:, 0] / (self.Ny * self.Nz)
        self.a_x = counts[:, 1] / (self.Ny * self.Nz * self.dx)
        # electrode.py:189-200
        self.resistance = 1
        self.capacitance = 1
        self.freq_0 = np.mean(self.vol_x) / np.mean(self.a_x * self.dx) / self.Nx ** 2
        if mode == "tau_e":
            self.frequency = np.array([self.freq_0 / 2, self.freq_0 / 4])
        elif mode == "nyquist":
            freq_range = self.freq_0 * 2 ** (np.arange(-3, 10, 0.5))
            self.frequency = freq_range[::-1]
        self.mode = mode
        self.Z_mean = compute_impedance(np.full(self.Nx, 1 / np.mean(self.vol_x)),
                                        np.full(self.Nx, np.mean(self.a_x * self.dx)), self.frequency)
        self.sum_iter = 0
        self.c_x = 0

    # ------------------------------------------------------------ reference surface
    @property
    def field(self):
        """The solver's complex128 field [1, Nx+2, Ny+2, Nz+2] on the device (None before solve)."""
        return self._field

    @field.setter
    def field(self, value):
        self._field = value

    @property
    def mask(self) -> torch.Tensor:
        """float64 [1, Nx, Ny, Nz] conductive mask (electrode.py:181-182)."""
        return (self._code >> 7).to(torch.float64)[None]

    @property
    def cond_nn(self) -> torch.Tensor:
        """float64 [1, Nx, Ny, Nz] conductive face neighbours, inlet counted 2 (electrode.py:248-251)."""
        return ((self._code & 0x7F) % 8).to(torch.float64)[None]

    @property
    def reac_nn(self) -> torch.Tensor:
        """float64 [1, Nx, Ny, Nz] reactive face neighbours (electrode.py:253-258)."""
        return ((self._code & 0x7F) // 8).to(torch.float64)[None]

    @property
    def cb(self):
        """[omega * even, omega * odd] chequerboards, float64 [Nx, Ny, Nz] (taufactor.py:218-225)."""
        a = torch.arange(self.Nx, device=self.device)[:, None, None]
        b = torch.arange(self.Ny, device=self.device)[None, :, None]
        c = torch.arange(self.Nz, device=self.device)[None, None, :]
        even = ((a + b + c) % 2 == 0).to(torch.float64)
        return [self.omega * even, self.omega * (1 - even)]

    def return_mask(self, img):
        mask = torch.zeros_like(img)
        mask[img == self.cond_label] = 1
        return mask

    def init_field(self, img):
        return None

    def init_conductive_neighbours(self, img):
        return None

    def count_neighbours(self, img, mask):
        """(cond_nn, reac_nn) of the solver's own volume (electrode.py:235-264)."""
        return self.cond_nn, self.reac_nn

    def _profile(self, frc) -> np.ndarray:
        """electrode.py:223-226: left_bc cosh(l (Nx - x)) / cosh(l Nx), l = sqrt(i frc
        mean(a_x[1:-1] dx) / mean(vol_x)), at the voxel centres."""
        x = np.arange(0, self.Nx) + 0.5
        lambda_0 = np.sqrt(1j * frc * np.mean(self.a_x[1:-1] * self.dx) / np.mean(self.vol_x))
        return self.left_bc * np.cosh(lambda_0 * (self.Nx - x)) / np.cosh(lambda_0 * self.Nx)

    def init_field_internal(self, mask=None):
        """Padded complex128 field [1, Nx+2, Ny+2, Nz+2] for the current frc
        (electrode.py:214-233); the conductive mask is the solver's own."""
        return self._fill(np.asarray(self._profile(self.frc), dtype=np.complex128)[None])

    def _fill(self, phi: np.ndarray) -> torch.Tensor:
        F = phi.shape[0]
        with torch.cuda.device(self.device):
            field = torch.empty((F, self.Nx + 2, self.Ny + 2, self.Nz + 2), dtype=torch.complex128,
                                device=self.device)
            phi_dev = torch.from_numpy(np.ascontiguousarray(phi, dtype=np.complex128)).to(self.device)
            check(self._lib.tf_impedance_fill(F, self.Nx, self.Ny, self.Nz, self._code.data_ptr(),
                                              phi_dev.data_ptr(), 2 * self.left_bc, field.data_ptr(),
                                              self._stream()), "tf_impedance_fill")
        return field

    def apply_boundary_conditions(self):
        """Default: Dirichlet in x, no flux in y and z (taufactor.py:91-93)."""

    def _check_field(self, field, n_freq):
        shape = (n_freq, self.Nx + 2, self.Ny + 2, self.Nz + 2)
        if (not isinstance(field, torch.Tensor) or field.dtype != torch.complex128 or tuple(field.shape) != shape
                or not field.is_contiguous() or field.device != self.device):
            raise ValueError(f"field must be a contiguous complex128 tensor of shape {shape} on {self.device}")

    def _advance(self, n: int, field=None, table=None, active=None, n_freq=1):
        field = self.field if field is None else field
        table = self._table if table is None else table
        self._check_field(field, n_freq)
        with torch.cuda.device(self.device):
            check(self._lib.tf_impedance_sweep(n_freq, self.Nx, self.Ny, self.Nz, self._periodic, field.data_ptr(),
                                               self._code.data_ptr(), table.data_ptr(),
                                               None if active is None else active.data_ptr(), float(self.omega),
                                               self.iter, n, self._stream()), "tf_impedance_sweep")

    def _reduce(self, field=None, n_freq=1):
        """(abs sums [F, Nx], inlet flux sums [F] complex, NaN cells [F]) of the field."""
        field = self.field if field is None else field
        self._check_field(field, n_freq)
        with torch.cuda.device(self.device):
            if self._abs.shape[0] != n_freq:
                self._abs = torch.empty((n_freq, self.Nx), dtype=torch.float64, device=self.device)
                self._influx = torch.empty(2 * n_freq, dtype=torch.float64, device=self.device)
                self._nan = torch.zeros(n_freq, dtype=torch.int32, device=self.device)
            check(self._lib.tf_impedance_metrics(n_freq, self.Nx, self.Ny, self.Nz, field.data_ptr(),
                                                 float(self.left_bc), self._abs.data_ptr(), self._influx.data_ptr(),
                                                 self._nan.data_ptr(), self._stream()), "tf_impedance_metrics")
            a = self._abs.cpu().numpy()
            q = self._influx.cpu().numpy().reshape(n_freq, 2)
            nan = self._nan.cpu().numpy()
        return a, q[:, 0] + 1j * q[:, 1], nan

    def _set_factor(self, frc):
        with torch.cuda.device(self.device):
            self._table.copy_(torch.from_numpy(factor_table(frc)))

    def calc_input_impedance(self):
        """left_bc / mean inlet flux, the flux 2 left_bc - 2 c over plane 0 (0 where c = 0)
        (electrode.py:324-330)."""
        _, q, _ = self._reduce()
        influx = np.array([q[0].real / (self.Ny * self.Nz) + 1j * (q[0].imag / (self.Ny * self.Nz))])
        return self.left_bc / influx[0]

    def _metrics_from(self, abs_sum, q, c_x_prev):
        """compute_metrics (electrode.py:379-392) on one frequency's sums: (c_av or None if it
        holds NaN, relative error, input impedance)."""
        area = self.Ny * self.Nz
        c_av = abs_sum / area
        c_av[self.vol_x > 0] /= self.vol_x[self.vol_x > 0]
        relative_error = np.array(np.max(np.abs(c_av - c_x_prev)) / (np.max(c_av) - np.min(c_av)))
        if np.any(np.isnan(c_av)):
            return None, relative_error, None
        influx = np.array([q.real / area + 1j * (q.imag / area)])
        return c_av, relative_error, self.left_bc / influx[0]

    def compute_metrics(self):
        """electrode.py:379-392 on float64 plane sums read back from the device."""
        a, q, _ = self._reduce()
        c_av, relative_error, z = self._metrics_from(a[0], q[0], self.c_x)
        if c_av is None:
            return np.expand_dims(0.0, axis=0), np.expand_dims(0.0, axis=0)
        self.c_x = c_av
        self.impedance[-1] = z
        tau = np.array(self.impedance[-1].real / self.Z_mean[-1].real)
        return np.expand_dims(tau, axis=0), np.expand_dims(relative_error, axis=0)

    def solve(self, iter_limit=10000, verbose=True, conv_crit=1e-3, plot_interval=10):
        """The frequency loop of electrode.py:266-322; returns None like the reference."""
        if verbose:
            torch.cuda.reset_peak_memory_stats(device=self.device)
        if verbose == "debug":
            self.tau_t = []
        self.impedance = []
        self.converged_freq = []
        self.taus = []
        self.frc = self.frequency[0] * self.resistance * self.capacitance
        self.field = self.init_field_internal()
        start = timer()
        for f in self.frequency:
            self.frc = f * self.resistance * self.capacitance
            if self._reduce()[2][0]:
                self.field = self.init_field_internal()
            self._set_factor(self.frc)
            self.impedance.append(0)
            self.converged = False
            self.tau = 0
            self.iter = 0
            while not self.converged and self.iter < iter_limit:
                n = min(100 - self.iter % 100, iter_limit - self.iter)
                self._advance(n)
                self.iter += n
                if self.iter % 100 == 0:
                    self.converged = self.check_convergence(verbose, conv_crit, plot_interval)
            self.converged_freq.append(self.converged)
            self.sum_iter += self.iter
            self.taus.append(self.tau)
        print(self.taus)
        torch.cuda.synchronize(self.device)
        self.walltime = timer() - start
        self._end_simulation(self.sum_iter, verbose)

    # ------------------------------------------------------------ frequency batch
    def solve_frequencies(self, frequencies=None, iter_limit=10000, conv_crit=1e-3):
        """Solve every frequency (default: ``self.frequency``) as an independent system, side by
        side in one set of launches, each from its own analytic profile and each stopped by the
        reference's rule (layer means of |c| and tau checked every 100 half-sweeps) or at
        iter_limit. No reference counterpart: the reference's loop warm-starts each frequency
        from the previous one, so its iteration counts (not the converged values) differ.

        Returns dict(frequency, impedance [F] complex, tau [F], iters [F], converged [F], field
        [F, Nx+2, Ny+2, Nz+2])."""
        freqs = np.asarray(self.frequency if frequencies is None else frequencies, dtype=np.float64).reshape(-1)
        F = freqs.shape[0]
        frcs = freqs * self.resistance * self.capacitance
        phi = np.stack([self._profile(frc) for frc in frcs]).astype(np.complex128)
        field = self._fill(phi)
        with torch.cuda.device(self.device):
            table = torch.from_numpy(np.stack([factor_table(frc) for frc in frcs])).to(self.device)
            active_h = np.ones(F, dtype=np.uint8)
            active = torch.from_numpy(active_h.copy()).to(self.device)
        iters = np.zeros(F, dtype=np.int64)
        conv = np.zeros(F, dtype=bool)
        c_x = [0] * F
        old_tau = np.zeros(F)
        tau = np.zeros(F)
        imp = np.zeros(F, dtype=np.complex128)
        saved_iter = self.iter
        it = 0
        try:
            while active_h.any() and it < iter_limit:
                n = min(100 - it % 100, iter_limit - it)
                self.iter = it
                self._advance(n, field=field, table=table, active=active, n_freq=F)
                it += n
                iters[active_h.astype(bool)] = it
                if it % 100:
                    continue
                a, q, _ = self._reduce(field=field, n_freq=F)
                changed = False
                for k in np.flatnonzero(active_h):
                    c_av, rel, z = self._metrics_from(a[k], q[k], c_x[k])
                    if c_av is None:
                        t, rel = 0.0, 0.0
                    else:
                        c_x[k] = c_av
                        imp[k] = z
                        t = z.real / self.Z_mean[-1].real
                    tau[k] = t
                    if not rel < conv_crit or not abs(t - old_tau[k]) < 2e-3:
                        old_tau[k] = t
                        continue
                    if t == 0:
                        tau[k] = np.inf
                    conv[k] = True
                    active_h[k] = 0
                    changed = True
                if changed:
                    with torch.cuda.device(self.device):
                        active.copy_(torch.from_numpy(active_h.copy()))
        finally:
            self.iter = saved_iter
        return dict(frequency=freqs, impedance=imp, tau=tau, iters=iters, converged=conv, field=field)


class PeriodicImpedanceSolver(ImpedanceSolver):
    """Impedance solver, periodic in y and z (electrode.py:369-402)."""

    _periodic = 1

    def apply_boundary_conditions(self):
        """electrode.py:398-402 on ``field`` (the sweeps copy the ghosts on the device)."""
        self.field[:, :, 0, :] = self.field[:, :, -2, :]
        self.field[:, :, -1, :] = self.field[:, :, 1, :]
        self.field[:, :, :, 0] = self.field[:, :, :, -2]
        self.field[:, :, :, -1] = self.field[:, :, :, 1]
