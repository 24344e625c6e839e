"""float32 CPU restatement of TauFactor's red-black SOR through-transport solve.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the checker for the CUDA path, never the
thing measured or shipped.

Everything here follows tldr-group/taufactor v1.2.1, ``taufactor/taufactor.py``:

* input handling        ``SORSolver._expand_to_4d``                :195-204
* default omega         ``SORSolver.__init__``                     :36-37
* padding               ``SORSolver._pad``                         :228-238
* initial field         ``ThroughTransportSolver.init_field``      :282-291
* neighbour counts      ``Solver.init_conductive_neighbours``      :402-410
                        ``PeriodicSolver.init_conductive_neighbours`` :493-499
                        ``AnisotropicSolver.init_conductive_neighbours`` :459-471
* harmonic faces        ``MultiPhaseSolver._harmonic_mean`` / ``init_conductive_neighbours``
                                                                   :577-604, periodic :626-650
* chequerboard          ``SORSolver._init_chequerboard``           :218-225
* half-sweep            ``SORSolver.solve`` loop body              :174-182
                        ``sum_weighted_neighbours``  :95-103, :473-478, :606-613
                        periodic ghost copy :501-505, :652-656
* flux / metrics        ``vertical_flux`` :412-419, :615-620; ``compute_metrics`` :293-331
* convergence           ``SORSolver.check_convergence``            :109-153
* electrode             ``ElectrodeSolver`` / ``PeriodicElectrodeSolver`` (taufactor/electrode.py:13-157):
                        masks :36-40, cosh initial field :42-50, neighbour counts :52-62 and
                        :135-150, reaction prefactor ``SORSolver.__init__`` :47-55, metrics :64-103;
                        impedance ``compute_impedance_batched`` (taufactor/utils.py:75-98)

The per-element float32 operation order is the reference's (left-to-right neighbour sums, one
IEEE rounding per operation, no fused multiply-add), so a half-sweep here is bitwise equal to the
reference's (up to the sign of zero). The only deliberate difference is in the metrics: the
per-layer means of the flux and of the field are accumulated in float64 here (the reference
reduces in float32); ``tests/test_oracle.py`` bounds the effect against the reference's goldens.
"""
from __future__ import annotations

import math

import numpy as np

from .percolation import spans_axis0

F32 = np.float32

KINDS = ("binary", "periodic", "anisotropic", "multiphase", "periodic_multiphase", "kappa", "periodic_kappa",
         "electrode", "periodic_electrode")


def expand_to_4d(img) -> np.ndarray:
    """ndarray -> [B, X, Y, Z] (taufactor.py:195-204)."""
    if not isinstance(img, np.ndarray):
        raise TypeError("Error: input image must be a NumPy array!")
    if img.ndim == 2:
        img = img[..., None]
    if img.ndim == 3:
        img = img[None, ...]
    if img.ndim != 4:
        raise ValueError("expected [B, X, Y, Z]")
    return img


def default_omega(nx: int) -> float:
    """Over-relaxation default 2 - pi/(1.5 Nx) in float64 (taufactor.py:36-37)."""
    return 2.0 - math.pi / (1.5 * nx)


def linear_profile(nx: int, top_bc: float = -0.5, bot_bc: float = 0.5) -> np.ndarray:
    """float32 profile of the initial field along x (taufactor.py:284-286).

    The reference builds it with ``torch.linspace`` in float32; the same library call is used
    here so the initial field agrees bit for bit.
    """
    import torch

    sh = 1 / (2 * nx)
    return torch.linspace(top_bc + sh, bot_bc - sh, nx, dtype=torch.float32).numpy()


def pad_volume(vol: np.ndarray, xvals=(0.0, 0.0)) -> np.ndarray:
    """Pad [B,X,Y,Z] by one voxel on every spatial face (taufactor.py:228-238).

    The x-faces take ``xvals``; the y/z faces (including their rims on the x-faces) are 0.
    """
    out = np.zeros((vol.shape[0],) + tuple(s + 2 for s in vol.shape[1:]), dtype=vol.dtype)
    out[:, 1:-1, 1:-1, 1:-1] = vol
    out[:, 0] = xvals[0]
    out[:, -1] = xvals[1]
    out[:, :, 0] = 0
    out[:, :, -1] = 0
    out[:, :, :, 0] = 0
    out[:, :, :, -1] = 0
    return out


def _roll_sum(t: np.ndarray, weights=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Sum of the 6 circular shifts of t over its spatial axes, axis-weighted."""
    s = np.zeros_like(t)
    for ax, w in zip((1, 2, 3), weights):
        for dr in (1, -1):
            r = np.roll(t, dr, axis=ax)
            s += r if w == 1.0 else r * F32(w)
    return s


def neighbour_counts(mask: np.ndarray, periodic: bool = False, weights=(1.0, 1.0, 1.0), xpad=(2.0, 2.0),
                     zero_inf: bool = True) -> np.ndarray:
    """Conductive-neighbour count nn, inf where solid or nn == 0.

    Dirichlet x-faces count twice because the conductor boundary sits half a voxel away
    (pad with 2: taufactor.py:402-410). Periodic variant wraps y,z (:493-499); anisotropic
    variant weights y,z neighbours by (dx/dy)^2, (dx/dz)^2 (:459-471).
    """
    m = mask.astype(F32)
    p = pad_volume(m, xpad)
    if periodic:
        p = p[:, :, 1:-1, 1:-1]
        nn = _roll_sum(p, weights)[:, 1:-1]
    else:
        nn = _roll_sum(p, weights)[:, 1:-1, 1:-1, 1:-1]
    nn = nn.copy()
    nn[m == 0] = np.inf
    if zero_inf:
        nn[nn == 0] = np.inf
    return nn


def electrode_prefactor(cond: np.ndarray, reac: np.ndarray, periodic: bool, dx: float):
    """Reactive-neighbour counts (electrode.py:52-62 / :143-150) and the reference's float32
    a_x [B,Nx], k_0 [B], vol_x [B,Nx] (taufactor.py:40-55). Computed with the same torch float32
    operations as the reference, so k_0 agrees to the last bit."""
    import torch

    B, X, Y, Z = cond.shape
    mask_t = torch.from_numpy(cond.astype(F32))
    vol_x = torch.mean(mask_t, (2, 3))
    r = torch.from_numpy(reac.astype(F32))
    rp = torch.nn.functional.pad(r, (0, 0, 0, 0, 1, 1) if periodic else (1, 1, 1, 1, 1, 1))
    s = torch.zeros_like(rp)
    for dim in range(1, 4):
        for dr in (1, -1):
            s += torch.roll(rp, dr, dim)
    reac_nn = s[:, 1:-1] if periodic else s[:, 1:-1, 1:-1, 1:-1]
    reac_nn[~torch.from_numpy(cond)] = 0.0
    a_x = torch.sum(reac_nn, (2, 3)) / (Y * Z * dx)
    k_0 = torch.mean(vol_x, 1) / torch.mean(a_x * dx, 1) / X ** 2
    return reac_nn.numpy(), a_x.numpy(), k_0.numpy(), vol_x.numpy()


def compute_impedance_batched(R: np.ndarray, C: np.ndarray, freq: np.ndarray) -> np.ndarray:
    """Transmission-line impedance [B,F] (taufactor/utils.py:75-98)."""
    bs, nx = R.shape
    w = freq[None, :].repeat(bs, axis=0) if freq.ndim == 1 else freq
    Z = np.full_like(w, 1e50, dtype=complex)
    for k in range(nx - 1, -1, -1):
        Z = R[:, k][:, None] + 1.0 / (1j * w * C[:, k][:, None] + 1.0 / Z)
    return Z


def harmonic_mean(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """2ab/(a+b) in float32, 0 where a+b == 0 (taufactor.py:577-583)."""
    den = a + b
    out = np.zeros_like(den)
    v = den > 0
    out[v] = F32(2) * a[v] * b[v] / den[v]
    return out


def diffusivity_map(labels: np.ndarray, ds: dict) -> np.ndarray:
    """Per-voxel float32 diffusivity from a label->D dict (taufactor.py:586-588)."""
    lab = labels.astype(F32)
    dmap = np.zeros_like(lab)
    for phase, d in ds.items():
        dmap[lab == F32(phase)] = F32(d)
    return dmap


def face_conductances(dmap: np.ndarray, periodic: bool = False):
    """Harmonic-mean face conductances D_x, D_y, D_z and the diagonal ``factor``.

    x ghost planes copy the adjacent voxel (taufactor.py:590-592); y/z ghosts are 0, or the
    opposite interior plane when periodic (:633-638). factor = sum of the 6 faces plus the
    boundary face once more on x = 0 and x = Nx-1, 0 -> inf (:598-603).
    """
    d = pad_volume(dmap, (0.0, 0.0))
    d[:, 0] = d[:, 1]
    d[:, -1] = d[:, -2]
    if periodic:
        d[:, :, 0, :] = d[:, :, -2, :]
        d[:, :, -1, :] = d[:, :, 1, :]
        d[:, :, :, 0] = d[:, :, :, -2]
        d[:, :, :, -1] = d[:, :, :, 1]
    dx = harmonic_mean(d[:, :-1, 1:-1, 1:-1], d[:, 1:, 1:-1, 1:-1])
    dy = harmonic_mean(d[:, 1:-1, :-1, 1:-1], d[:, 1:-1, 1:, 1:-1])
    dz = harmonic_mean(d[:, 1:-1, 1:-1, :-1], d[:, 1:-1, 1:-1, 1:])
    factor = dx[:, :-1] + dx[:, 1:] + dy[:, :, :-1] + dy[:, :, 1:] + dz[:, :, :, :-1] + dz[:, :, :, 1:]
    factor[:, 0] += dx[:, 0]
    factor[:, -1] += dx[:, -1]
    factor[factor == 0] = np.inf
    return dx, dy, dz, factor


def chequerboard(shape3, omega: float):
    """float32 omega-weighted colour masks; colour 0 is (i+j+k) even (taufactor.py:218-225)."""
    a, b, c = np.meshgrid(*(np.arange(n) for n in shape3), indexing="ij")
    even = ((a + b + c) % 2 == 0).astype(np.float64)
    return [(omega * even).astype(F32), (omega * (1 - even)).astype(F32)]


class OracleSolve:
    """One batched through-transport solve, restated from the reference.

    ``kind`` selects the reference class being restated:
    ``binary`` (Solver), ``periodic`` (PeriodicSolver), ``anisotropic`` (AnisotropicSolver),
    ``multiphase`` (MultiPhaseSolver), ``periodic_multiphase`` (PeriodicMultiPhaseSolver).
    """

    top_bc, bot_bc = -0.5, 0.5

    def __init__(self, img, kind="binary", omega=None, D_0=1.0, diffusivities=None,
                 spacing=None, conductive_label=1, reactive_label=0):
        if kind not in KINDS:
            raise ValueError(f"unknown kind {kind}")
        self.kind = kind
        self.cpu_img = expand_to_4d(img)
        self.batch_size, self.Nx, self.Ny, self.Nz = self.cpu_img.shape
        if omega is None:
            omega = default_omega(self.Nx)
        self.omega = omega
        self.periodic = kind in ("periodic", "periodic_multiphase", "periodic_kappa", "periodic_electrode")
        self.multiphase = kind in ("multiphase", "periodic_multiphase", "kappa", "periodic_kappa")
        self.electrode = kind in ("electrode", "periodic_electrode")
        img32 = self.cpu_img.astype(F32)
        if self.electrode:
            self._init_electrode(img32, omega, spacing, conductive_label, reactive_label)
            return
        if kind in ("kappa", "periodic_kappa"):
            # per-voxel float32 diffusivity given directly (MultiPhaseSolver's map, :586-588)
            self.Ds = {}
            self.conductive_labels = [1]
            dmap = img32
            self.kappa = img32
            mask = (dmap > 0).astype(F32)
            self.D_x, self.D_y, self.D_z, self.factor = face_conductances(dmap, self.periodic)
            self.cpu_img = (dmap > 0).astype(np.uint8)
        elif self.multiphase:
            ds = dict({0: 0, 1: 1} if diffusivities is None else diffusivities)
            for lbl in np.unique(self.cpu_img):
                if lbl not in ds:
                    ds[int(lbl)] = 0.0
            self.Ds = ds
            self.conductive_labels = [lbl for lbl, d in ds.items() if d > 0]
            mask = np.isin(img32, np.array(self.conductive_labels, dtype=F32)).astype(F32) \
                if self.conductive_labels else np.zeros_like(img32)
            self.D_x, self.D_y, self.D_z, self.factor = face_conductances(
                diffusivity_map(self.cpu_img, ds), self.periodic)
        else:
            self.conductive_labels = [1]
            mask = img32
            w = (1.0, 1.0, 1.0)
            if kind == "anisotropic":
                dx, dy, dz = spacing
                self.Ky, self.Kz = (dx / dy) ** 2, (dx / dz) ** 2
                w = (1.0, self.Ky, self.Kz)
            self.factor = neighbour_counts(mask, self.periodic, w)
        self.mask = mask
        # vol_x as float64 means of the mask (the reference takes a float32 torch mean, :42)
        self.vol_x = mask.astype(np.float64).mean(axis=(2, 3))
        prof = linear_profile(self.Nx, self.top_bc, self.bot_bc)
        self.field = pad_volume(mask * prof[None, :, None, None],
                                (2 * self.top_bc, 2 * self.bot_bc)).astype(F32)
        self.cb = chequerboard((self.Nx, self.Ny, self.Nz), omega)
        if kind in ("kappa", "periodic_kappa"):
            self.D_0 = D_0
            self.D_mean = img32.astype(np.float64).mean(axis=(1, 2, 3))
        elif self.multiphase:
            vf = {int(p): np.mean(self.cpu_img == p, axis=(1, 2, 3)) for p in np.unique(self.cpu_img)}
            self.D_0 = D_0
            self.D_mean = np.sum([vf[z] * self.Ds.get(z, 0.0) for z in vf], axis=0)
        else:
            self.D_0 = D_0
            self.D_mean = self.vol_x.mean(axis=1)
        self.iter = 0
        self.converged = False
        self.old_tau = 0
        self.tau = self.tau_x = self.D_eff = None

    def _init_electrode(self, img32, omega, spacing, cond_label, reac_label):
        """ElectrodeSolver / PeriodicElectrodeSolver set-up (electrode.py:18-62, taufactor.py:40-55)."""
        self.left_bc, self.electrode_bc = 1.0, 0.0
        self.dx = spacing or 1
        cond = img32 == F32(cond_label)
        reac = (img32 == F32(reac_label)) & ~cond
        mask = cond.astype(F32)
        nn = neighbour_counts(mask, self.periodic, xpad=(2.0, 0.0), zero_inf=False)
        reac_nn, self.a_x, self.k_0, self.vol_x = electrode_prefactor(cond, reac, self.periodic, self.dx)
        factor = nn + reac_nn * self.k_0[:, None, None, None]
        factor[factor == 0] = np.inf
        self.factor = factor.astype(F32)
        self.mask = mask
        self.conductive_labels = [cond_label]
        x = np.arange(self.Nx) + 0.5
        c_init = self.electrode_bc + (self.left_bc - self.electrode_bc) * np.cosh(1 - x / self.Nx) / np.cosh(1)
        vec = c_init.astype(F32)
        self.field = pad_volume(mask * vec[None, :, None, None], (2 * self.left_bc, 0.0)).astype(F32)
        self.cb = chequerboard((self.Nx, self.Ny, self.Nz), omega)
        self.c_x = 0
        self.iter = 0
        self.converged = False
        self.old_tau = 0
        self.tau = self.tau_x = self.D_eff = None

    def electrode_layer_means(self, dtype=F32):
        """float64 per-layer means of ElectrodeSolver's fluxes [B,Nx] and of the field [B,Nx]
        (electrode.py:65, :70-74): plane 0 (left_bc - c)/0.5, plane x > 0 c[x-1] - c[x], 0 where
        c or c[x-1] is 0. The fluxes are formed in float32 like the reference's, or in float64
        (dtype=np.float64) for a float64 field."""
        f = self.field
        c = f[:, 1:-1, 1:-1, 1:-1]
        cm = f[:, :-2, 1:-1, 1:-1]
        fl = (-c + cm).astype(dtype)
        fl[:, 0] = (dtype(self.left_bc) - c[:, 0]) / dtype(0.5)
        fl[c == 0] = 0
        fl[cm == 0] = 0
        return fl.astype(np.float64).mean(axis=(2, 3)), c.astype(np.float64).mean(axis=(2, 3))

    def electrode_metrics(self, dtype=F32):
        """electrode.py:64-103 on the float64 layer means."""
        fluxes, c_raw = self.electrode_layer_means(dtype)
        vol_x = self.vol_x
        c_x = np.divide(c_raw, vol_x, out=np.zeros(c_raw.shape), where=vol_x != 0)
        rel = np.max(np.abs(c_x - self.c_x), axis=1)
        self.c_x = c_x
        f1 = np.concatenate((2 * (self.left_bc - c_x[:, :1]), (-c_x[:, 1:] + c_x[:, :-1])), axis=1)
        f1[:, 1:][vol_x[:, 1:] == 0] = 0
        f1[:, 1:][vol_x[:, :-1] == 0] = 0
        eps = np.concatenate((vol_x[:, :1], 0.5 * (vol_x[:, :-1] + vol_x[:, 1:])), axis=1)
        self.tau_x = np.divide(eps * f1, fluxes, out=np.full_like(f1, np.nan), where=fluxes != 0)
        fluxes[:, :-1] -= fluxes[:, 1:]
        self.k_x = np.divide(fluxes, c_x - self.electrode_bc, out=np.zeros_like(c_x),
                             where=(c_x - self.electrode_bc) != 0) / self.k_0[:, None]
        freq = np.mean(eps, axis=1, keepdims=True) / np.mean(self.a_x * self.dx, axis=1, keepdims=True) / self.Nx ** 2 * 2 ** -3
        R = self.tau_x / eps
        R[eps == 0] = 1e30
        R[np.isnan(self.tau_x)] = 1e30
        z_sim = compute_impedance_batched(R, self.a_x * self.dx, freq)
        r_id = 1 / np.mean(eps, axis=1)[:, None].repeat(self.Nx, axis=1)
        c_id = np.mean(self.a_x * self.dx, axis=1)[:, None].repeat(self.Nx, axis=1)
        z_id = compute_impedance_batched(r_id, c_id, freq)
        return z_sim[:, 0].real / z_id[:, 0].real, rel

    # -------------------------------------------------------------- half-sweep
    def apply_boundary_conditions(self):
        """Periodic ghost planes from the opposite interior planes (taufactor.py:501-505)."""
        if self.periodic:
            f = self.field
            f[:, :, 0, :] = f[:, :, -2, :]
            f[:, :, -1, :] = f[:, :, 1, :]
            f[:, :, :, 0] = f[:, :, :, -2]
            f[:, :, :, -1] = f[:, :, :, 1]

    def neighbour_sum(self) -> np.ndarray:
        f = self.field
        if self.multiphase:
            return (f[:, 2:, 1:-1, 1:-1] * self.D_x[:, 1:] + f[:, :-2, 1:-1, 1:-1] * self.D_x[:, :-1]
                    + f[:, 1:-1, 2:, 1:-1] * self.D_y[:, :, 1:] + f[:, 1:-1, :-2, 1:-1] * self.D_y[:, :, :-1]
                    + f[:, 1:-1, 1:-1, 2:] * self.D_z[:, :, :, 1:]
                    + f[:, 1:-1, 1:-1, :-2] * self.D_z[:, :, :, :-1])
        if self.kind == "anisotropic":
            ky, kz = F32(self.Ky), F32(self.Kz)
            return (f[:, 2:, 1:-1, 1:-1] + f[:, :-2, 1:-1, 1:-1]
                    + ky * (f[:, 1:-1, 2:, 1:-1] + f[:, 1:-1, :-2, 1:-1])
                    + kz * (f[:, 1:-1, 1:-1, 2:] + f[:, 1:-1, 1:-1, :-2]))
        return (f[:, 2:, 1:-1, 1:-1] + f[:, :-2, 1:-1, 1:-1] + f[:, 1:-1, 2:, 1:-1]
                + f[:, 1:-1, :-2, 1:-1] + f[:, 1:-1, 1:-1, 2:] + f[:, 1:-1, 1:-1, :-2])

    def half_sweep(self, n: int = 1, rhs=None):
        """n reference iterations (each one colour): taufactor.py:174-182.

        ``rhs`` (float32 [B,X,Y,Z], no reference counterpart) is added to the neighbour sum, which
        turns the iteration into SOR for A e = rhs; it restates the correction solve of the
        FP64 defect correction.
        """
        for _ in range(n):
            self.apply_boundary_conditions()
            inc = self.neighbour_sum()
            if rhs is not None:
                inc += rhs
            inc /= self.factor
            inc -= self.field[:, 1:-1, 1:-1, 1:-1]
            inc *= self.cb[self.iter % 2]
            self.field[:, 1:-1, 1:-1, 1:-1] += inc
            self.iter += 1

    # -------------------------------------------------------------- metrics
    def vertical_flux(self) -> np.ndarray:
        f = self.field
        d = f[:, 2:-1, 1:-1, 1:-1] - f[:, 1:-2, 1:-1, 1:-1]
        if self.multiphase:
            return self.D_x[:, 1:-1] * d
        d = d.copy()
        d[self.factor[:, :-1] > 8] = 0
        d[self.factor[:, 1:] > 8] = 0
        return d

    def layer_means(self):
        """float64 per-layer means of the x-flux [B,Nx-1] and of the field [B,Nx]."""
        flux = self.vertical_flux().astype(np.float64).mean(axis=(2, 3))
        cx = self.field[:, 1:-1, 1:-1, 1:-1].astype(np.float64).mean(axis=(2, 3))
        return flux, cx

    def compute_metrics(self):
        """tau, relative error and D_eff from the layer fluxes (taufactor.py:293-331)."""
        if self.electrode:
            return self.electrode_metrics()
        self.flux_1d, c_x = self.layer_means()
        return metrics_from_layers(self, self.flux_1d, c_x)

    def check_convergence(self, conv_crit: float) -> bool:
        """taufactor.py:109-153 (without the plotting branches)."""
        self.tau, rel = self.compute_metrics()
        if not np.all(rel < conv_crit):
            self.old_tau = self.tau
            return False
        if not np.max(np.abs(self.tau - self.old_tau)) < 2e-3:
            self.old_tau = self.tau
            return False
        self.tau[self.tau == 0] = np.inf
        return True

    def solve(self, iter_limit=10000, conv_crit=1e-2):
        """The reference's solve loop: checks every 100 half-sweeps (taufactor.py:156-191)."""
        while not self.converged and self.iter < iter_limit:
            self.half_sweep(1)
            if self.iter % 100 == 0:
                self.converged = self.check_convergence(conv_crit)
        return self.tau if self.tau_x is None else self.tau_x


def metrics_from_layers(s, flux_1d: np.ndarray, c_x_raw: np.ndarray):
    """Host-side metric arithmetic on the per-layer means (taufactor.py:297-331).

    ``s`` provides Nx, D_mean, D_0, vol_x, batch_size, cpu_img, conductive_labels; it receives
    c_x, tau_x and D_eff. Returns (tau, relative_error).
    """
    fl_max = flux_1d.max(axis=1)
    fl_min = flux_1d.min(axis=1)
    mean_fl = flux_1d.mean(axis=1)
    rel = np.divide(fl_max - fl_min, fl_max, out=np.full_like(fl_max, np.nan), where=fl_max != 0)
    d_rel = mean_fl * s.Nx / abs(s.top_bc - s.bot_bc)
    tau = np.divide(s.D_mean, d_rel, out=np.full_like(d_rel, np.nan), where=d_rel != 0)
    c_x = np.divide(c_x_raw, s.vol_x, out=np.zeros_like(s.vol_x), where=s.vol_x != 0)
    s.c_x = c_x
    dc = c_x[:, 1:] - c_x[:, :-1]
    dc[s.vol_x[:, 1:] == 0] = 0
    dc[s.vol_x[:, :-1] == 0] = 0
    eps = 0.5 * (s.vol_x[:, :-1] + s.vol_x[:, 1:])
    s.tau_x = np.divide(eps * dc, flux_1d, out=np.full_like(dc, np.nan), where=flux_1d != 0)
    for b in range(s.batch_size):
        if fl_min[b] == 0 or fl_max[b] == 0 or mean_fl[b] == 0:
            if not spans_axis0(np.isin(s.cpu_img[b], s.conductive_labels)):
                rel[b] = 0
                d_rel[b] = 0
                tau[b] = 0
                s.tau_x[b, :] = 0
    rel[np.isnan(mean_fl)] = 0
    s.D_eff = s.D_0 * d_rel
    return tau, rel
