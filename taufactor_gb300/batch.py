"""Batched solve of many binary volumes of uneven shapes on one GPU.

The reference batches only volumes of one shape along a leading axis, and the whole batch
iterates until its slowest member converges (taufactor/taufactor.py:30-31, :143). Here every
volume keeps its own shape, buffers and convergence state:

* one launch of the fused sweep per tile class advances all still-active volumes by 4
  half-sweeps; volumes whose z-extent is a multiple of 128 use 16 x 128 tiles, those whose
  y-extent is a multiple of 32 use 32 x 64, the others 16 x 64 (rows x z-cells), and the
  classes run on their own streams between checks. A work list (tile columns
  split into x-chunks) holds only the volumes still active when the host last looked, and when
  few remain their chunks get shorter so that they still spread over the SMs (a volume's result
  does not depend on its tile class or on how its columns are chunked);
* every 100 half-sweeps the per-volume layer sums and the reference's convergence decision
  (taufactor.py:109-153, :293-331) run on the device and set a per-volume status;
* two such check intervals (50 sweep launches, two layer-sum and two decision launches) are
  captured once as a CUDA graph and replayed; the host reads the status flags between replays
  and only steps in for a volume whose layer flux is exactly zero (the percolation test of
  taufactor.py:318-327 runs on the host, as in the reference).

Each volume's result equals what ``Solver`` / ``PeriodicSolver`` return for it alone, except
that a volume paused for the percolation test skips one tau update. Optional FP64 defect
correction (``refine=True``) then runs for all volumes together: shared launches of the
correction sweeps, each volume stopping at its own tolerance.
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from timeit import default_timer as timer

import numpy as np
import torch

from . import _capi
from ._capi import (TF_BATCH_ACTIVE, TF_BATCH_CONVERGED, TF_BATCH_NEEDS_HOST, TF_KIND_BINARY, TF_PERIODIC_Y,
                    TF_PERIODIC_Z, TfBatchState, TfGeom, TfOperator, check)
from .percolation import spans_x
from .solvers import layer_metrics, unique_labels

INTERVAL = 100  # half-sweeps between convergence checks (taufactor.py:184-185)
_CAPTURE_LOCK = threading.Lock()
CHUNK = 32  # planes per work item of the batched sweep
MIN_CHUNK = 8  # shortest x-chunk when few volumes remain (each chunk streams 2 K extra planes)
RECOMPACT = 0.75  # rebuild the work list (and re-capture the graph) below this share of items


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class VolumeResult:
    """Outcome for one volume, with the attributes of the reference solver it stands for."""

    top_bc, bot_bc = -0.5, 0.5

    def __init__(self, img: np.ndarray, periodic: bool):
        self.cpu_img = img[None]
        self.batch_size, self.Nx, self.Ny, self.Nz = self.cpu_img.shape
        self.periodic = periodic
        self.conductive_labels = [1]
        mask = self.cpu_img == 1
        self.vol_x = mask.mean(axis=(2, 3), dtype=np.float64)
        self.D_mean = np.mean(self.vol_x, axis=1)
        self.D_0 = 1
        self.iter = 0
        self.converged = False
        self.tau = self.D_eff = self.tau_x = self.c_x = self.flux_1d = None
        self.residual_history = None


class BatchSolve:
    """Solve binary volumes of any shapes together.

    volumes   sequence of 3-D uint8/bool/int arrays with labels in {0, 1} (1 = conductive)
    periodic  bool or one bool per volume: PeriodicSolver (periodic y, z) instead of Solver
    omega     None (each volume's reference default 2 - pi/(1.5 Nx)), a float, or one per volume
    """

    def __init__(self, volumes, periodic=False, omega=None, device="cuda"):
        self.device = torch.device(device)
        if self.device.type != "cuda" or not torch.cuda.is_available():
            raise RuntimeError("BatchSolve runs on CUDA devices only")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        vols = [np.asarray(v) for v in volumes]
        n = len(vols)
        if n == 0:
            raise ValueError("no volumes")
        per = list(periodic) if isinstance(periodic, (list, tuple, np.ndarray)) else [bool(periodic)] * n
        om = list(omega) if isinstance(omega, (list, tuple, np.ndarray)) else [omega] * n
        if len(per) != n or len(om) != n:
            raise ValueError("periodic / omega must give one entry per volume")
        self.lib = lib = _capi.load()
        self.n = n
        self.results = []
        self.geoms = (TfGeom * n)()
        self.ops = (TfOperator * n)()
        self.fa, self.fb, self.codes = [], [], []
        ty, tz, kk = C.c_int(), C.c_int(), C.c_int()
        lib.tf_batch_tile(C.byref(ty), C.byref(tz), C.byref(kk))
        self.k = kk.value
        self._nx, self._tiles, self._cls = [], [], []
        flux_off, csum_off, d_mean = [], [], []
        nf = nc = 0
        with torch.cuda.device(self.device):
            self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
            for v, img in enumerate(vols):
                if img.ndim != 3:
                    raise ValueError("every volume must be 3-D")
                u = unique_labels(img)
                if len(u) > 2 or u.max() not in (0, 1) or u.min() not in (0, 1):
                    raise ValueError(f"volume {v}: labels must be 0/1, got {u}")
                res = VolumeResult(img, per[v])
                self.results.append(res)
                nx, ny, nz = img.shape
                pflag = (TF_PERIODIC_Y | TF_PERIODIC_Z) if per[v] else 0
                g = self.geoms[v]
                check(lib.tf_geometry(1, nx, ny, nz, pflag, C.byref(g)), "tf_geometry")
                if not g.tiled:
                    raise _capi.TfError(_capi.TF_ERR_UNSUPPORTED,
                                        f"BatchSolve volume {v} {img.shape}: periodic faces must be even and >= 16")
                op = self.ops[v]
                op.kind = TF_KIND_BINARY
                op.periodic = pflag
                # tile class (rows x z-cells): 16 x 128 where it covers the z-extent exactly, else
                # 32 x 64 where that covers the y-extent, else 16 x 64
                cls = 1 if nz % (2 * tz.value) == 0 else (2 if ny % (2 * ty.value) == 0 else 0)
                op.tile = cls
                w = om[v] if om[v] is not None else 2 - math.pi / (1.5 * nx)
                op.omega = float(np.float32(w))
                op.ghost_lo, op.ghost_hi = 2 * res.top_bc, 2 * res.bot_bc
                op.ky = op.kz = 1.0
                for i in range(256):
                    op.divisor[i] = float(i) if 1 <= i <= 8 else np.inf
                code = torch.empty(g.code_bytes, dtype=torch.uint8, device=self.device)
                fa = torch.empty(g.field_elems, dtype=torch.float32, device=self.device)
                fb = torch.zeros(g.field_elems, dtype=torch.float32, device=self.device)
                sh = 1 / (2 * nx)
                prof = torch.linspace(res.top_bc + sh, res.bot_bc - sh, nx, dtype=torch.float32).to(self.device)
                phase = torch.from_numpy(np.ascontiguousarray(img == 1, dtype=np.uint8)).to(self.device)
                check(lib.tf_pack(C.byref(g), C.byref(op), _ptr(phase), _ptr(prof), _ptr(code), _ptr(fa),
                                  self._stream()), "tf_pack")
                self.fa.append(fa)
                self.fb.append(fb)
                self.codes.append(code)
                tyc, tzc = ty.value * (2 if cls == 2 else 1), tz.value * (2 if cls == 1 else 1)
                self._tiles.append(((ny + tyc - 1) // tyc) * ((nz + tzc - 1) // tzc))
                self._nx.append(nx)
                self._cls.append(cls)
                flux_off.append(nf)
                csum_off.append(nc)
                nf += max(nx - 1, 1)
                nc += nx
                d_mean.append(float(res.D_mean[0]))
            self._sms = torch.cuda.get_device_properties(self.device).multi_processor_count
            self._work_cache, self._plane_cache = {}, {}
            self._set_work(tuple(range(n)))
            self._side = [None, torch.cuda.Stream(self.device), torch.cuda.Stream(self.device)]  # classes 1, 2
            self.flux = torch.zeros(nf, dtype=torch.float64, device=self.device)
            self.csum = torch.zeros(nc, dtype=torch.float64, device=self.device)
            self.flux_off, self.csum_off = flux_off, csum_off
            self.desc = torch.empty(int(lib.tf_batch_desc_bytes(n)), dtype=torch.uint8, device=self.device)
            P = C.c_void_p * n
            check(lib.tf_batch_describe(n, self.geoms, self.ops, P(*[_ptr(t) for t in self.fa]),
                                        P(*[_ptr(t) for t in self.fb]), P(*[_ptr(t) for t in self.codes]),
                                        (C.c_int64 * n)(*flux_off), (C.c_int64 * n)(*csum_off),
                                        (C.c_double * n)(*d_mean), _ptr(self.err), _ptr(self.desc)), "tf_batch_describe")
            i32 = dict(dtype=torch.int32, device=self.device)
            f64 = dict(dtype=torch.float64, device=self.device)
            self.status = torch.zeros(n, **i32)
            self.perc = torch.zeros(n, **i32)
            self.conv_iter = torch.zeros(n, **i32)
            self.conv_parity = torch.zeros(n, **i32)
            self.old_tau = torch.zeros(n, **f64)
            self.tau = torch.zeros(n, **f64)
            self.rel = torch.zeros(n, **f64)
            self.d_rel = torch.zeros(n, **f64)
            self.iter_base = torch.zeros(1, **i32)
        self.state = TfBatchState(_ptr(self.status), _ptr(self.perc), _ptr(self.conv_iter), _ptr(self.conv_parity),
                                  _ptr(self.old_tau), _ptr(self.tau), _ptr(self.rel), _ptr(self.d_rel),
                                  _ptr(self.iter_base))
        self.iter_offset = np.zeros(n, dtype=np.int64)
        self._final_in_b = np.zeros(n, dtype=bool)
        self.graph = None
        self._rhs = None
        self.c64 = None
        self.walltime = 0.0

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    # ---------------------------------------------------------------- work lists
    def _work_for(self, vols):
        """Work items (volume, tile, x0, x1) of the volumes `vols` per tile class: a pair of
        (int32 device tensor or None, count). Columns split into x-chunks of about CHUNK planes,
        so that items of large and small volumes take about equally long; when the items would
        not fill the SMs twice over, the chunks shrink (down to MIN_CHUNK planes) to spread the
        remaining volumes."""
        key = tuple(int(v) for v in vols)
        hit = self._work_cache.get(key)
        if hit is not None:
            return hit
        base = [max(1, round(self._nx[v] / CHUNK)) for v in key]
        total = sum(b * self._tiles[v] for b, v in zip(base, key))
        target = 2 * self._sms
        items = ([], [], [])
        for b, v in zip(base, key):
            nx, nch = self._nx[v], b
            if 0 < total < target:
                nch = min(max(1, nx // MIN_CHUNK), -(-b * target // total))
            bounds = [(c * nx) // nch for c in range(nch + 1)]
            items[self._cls[v]].extend((v, t, bounds[c], bounds[c + 1]) for t in range(self._tiles[v])
                                       for c in range(nch))
        hit = tuple((torch.tensor(it, dtype=torch.int32, device=self.device).reshape(-1) if it else None, len(it))
                    for it in items)
        self._work_cache[key] = hit
        return hit

    def _planes_for(self, vols):
        key = tuple(int(v) for v in vols)
        hit = self._plane_cache.get(key)
        if hit is None:
            planes = [(v, x) for v in key for x in range(self._nx[v])]
            hit = (torch.tensor(planes, dtype=torch.int32, device=self.device).reshape(-1), len(planes))
            self._plane_cache[key] = hit
        return hit

    def _set_work(self, vols):
        self.works = self._work_for(vols)
        self.n_work = sum(nw for _, nw in self.works)
        self.planes, self.n_planes = self._planes_for(vols)
        self._work_vols = set(int(v) for v in vols)

    def _compact(self, status) -> bool:
        """Shrink the work lists to the active volumes when that drops enough items (or when a
        volume resumed from a pause is missing from them); True if they changed."""
        act = tuple(np.flatnonzero(status == TF_BATCH_ACTIVE))
        if not act:
            return False
        w = self._work_for(act)
        if set(act) <= self._work_vols and sum(nw for _, nw in w) > RECOMPACT * self.n_work:
            return False
        self._set_work(act)
        return True

    # ---------------------------------------------------------------- device steps
    def _interval(self, interval: int, start_in_b: int, conv_crit: float):
        """100 half-sweeps of every active volume, then layer sums and the decision."""
        lib, st = self.lib, self._stream()
        main = torch.cuda.current_stream(self.device)
        # classes 1 and 2 sweep on their own streams meanwhile (volumes are independent)
        side = [c for c in (1, 2) if self.works[c][1]]
        for c in side:
            self._side[c].wait_stream(main)
        parity = start_in_b
        for _ in range(INTERVAL // self.k):
            for c, (w, nw) in enumerate(self.works):
                if nw:
                    stream = st if c == 0 else self._side[c].cuda_stream
                    check(lib.tf_batch_advance_tile(_ptr(self.desc), _ptr(w), nw, _ptr(self.status), parity, c,
                                                    stream), "tf_batch_advance_tile")
            parity ^= 1
        for c in side:
            main.wait_stream(self._side[c])
        check(lib.tf_batch_layer_sums(_ptr(self.desc), _ptr(self.planes), self.n_planes, _ptr(self.status), parity,
                                      _ptr(self.flux), _ptr(self.csum), st), "tf_batch_layer_sums")
        check(lib.tf_batch_check(_ptr(self.desc), self.n, _ptr(self.flux), self.state, float(conv_crit), interval,
                                 parity, st), "tf_batch_check")
        return parity

    def _pair(self, conv_crit: float):
        """Two intervals (an even number of launches, so the fields return to buffer A)."""
        p = self._interval(0, 0, conv_crit)
        p = self._interval(1, p, conv_crit)
        check(self.lib.tf_batch_tick(_ptr(self.iter_base), 2 * INTERVAL, self._stream()), "tf_batch_tick")
        assert p == 0

    def _capture(self, conv_crit: float):
        # one capture at a time in the process, checked against this thread's calls only, so the
        # batches of a MultiDeviceBatchSolve (one host thread each) may capture and read back
        # their status flags concurrently
        g = torch.cuda.CUDAGraph()
        with _CAPTURE_LOCK:
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(side):
                with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
                    self._pair(conv_crit)
            torch.cuda.current_stream(self.device).wait_stream(side)
        return g

    def _resolve_paused(self, status: np.ndarray, it: int):
        """Percolation test for volumes paused on a zero layer flux (taufactor.py:318-327)."""
        conv_iter = self.conv_iter.cpu().numpy()
        parity = self.conv_parity.cpu().numpy()
        for v in np.nonzero(status == TF_BATCH_NEEDS_HOST)[0]:
            res = self.results[v]
            if spans_x(res.cpu_img[0] == 1):
                self.perc[v] = 1
                # resume: the others advanced in lockstep meanwhile; realign the buffer parity
                # (graphs always start from buffer A) and remember the skipped half-sweeps
                if parity[v]:
                    self.fa[v].copy_(self.fb[v])
                self.iter_offset[v] += it - conv_iter[v]
                self.status[v] = TF_BATCH_ACTIVE
            else:
                print(f"Warning: volume {v} has no percolating path!")
                self.perc[v] = 2
                self.status[v] = TF_BATCH_CONVERGED

    # ---------------------------------------------------------------- public
    def solve(self, iter_limit: int = 10000, conv_crit: float = 1e-2, graph: bool = True, refine=False,
              poll: int = 2, verbose: bool = False):
        """Iterate every volume to the reference's convergence rule or iter_limit (rounded down
        to a multiple of 200); returns the list of VolumeResult.

        poll: graph replays (200 half-sweeps each) between two reads of the status flags.
        """
        limit = (iter_limit // (2 * INTERVAL)) * 2 * INTERVAL
        start = timer()
        self.c64 = None
        with torch.cuda.device(self.device):
            if self._compact(self.status.cpu().numpy()):
                self.graph = None
            if graph and self.graph is None:
                self.graph = self._capture(conv_crit)
                self._graph_crit = conv_crit
            if graph and self._graph_crit != conv_crit:
                self.graph = self._capture(conv_crit)
                self._graph_crit = conv_crit
            it = 0
            while it < limit:
                n_rep = min(poll, (limit - it) // (2 * INTERVAL))
                for _ in range(n_rep):
                    if graph:
                        self.graph.replay()
                    else:
                        self._pair(conv_crit)
                it += n_rep * 2 * INTERVAL
                status = self.status.cpu().numpy()
                if (status == TF_BATCH_NEEDS_HOST).any():
                    self._resolve_paused(status, it)
                    status = self.status.cpu().numpy()
                if verbose:
                    print(f"half-sweeps {it}: {int((status == TF_BATCH_ACTIVE).sum())} of {self.n} active")
                if not (status == TF_BATCH_ACTIVE).any():
                    break
                if self._compact(status) and graph:
                    self.graph = self._capture(conv_crit)
            if int(self.err.item()):
                raise _capi.TfError(int(self.err.item()), "tf_batch_advance (device)")
            self._collect(it)
            if refine:
                self.refine(**(refine if isinstance(refine, dict) else {}))
        torch.cuda.synchronize(self.device)
        self.walltime = timer() - start
        return self.results

    def _collect(self, it: int):
        status = self.status.cpu().numpy()
        conv_iter = self.conv_iter.cpu().numpy()
        parity = self.conv_parity.cpu().numpy()
        flux = self.flux.cpu().numpy()
        csum = self.csum.cpu().numpy()
        for v, res in enumerate(self.results):
            nx = res.Nx
            area = float(res.Ny * res.Nz)
            res.converged = bool(status[v] == TF_BATCH_CONVERGED)
            res.iter = int(conv_iter[v] - self.iter_offset[v]) if res.converged else int(it - self.iter_offset[v])
            # the field the metrics were taken from: buffer B if the decision saw it there
            self._final_in_b[v] = bool(parity[v]) if res.converged else False
            res.flux_1d = flux[self.flux_off[v]:self.flux_off[v] + nx - 1][None] / area
            c_x = csum[self.csum_off[v]:self.csum_off[v] + nx][None] / area
            if self.perc[v].item() == 2:
                res.flux_1d = np.zeros_like(res.flux_1d)
            tau, _ = layer_metrics(res, res.flux_1d, c_x)
            res.tau = np.where(tau == 0, np.inf, tau) if res.converged else tau

    def field(self, v: int) -> torch.Tensor:
        """Volume v's field in the reference's padded layout [1,Nx+2,Ny+2,Nz+2]."""
        res = self.results[v]
        buf = self.fb[v] if self._final_in_b[v] else self.fa[v]
        out = torch.empty((1, res.Nx + 2, res.Ny + 2, res.Nz + 2), dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            check(self.lib.tf_unpack(C.byref(self.geoms[v]), C.byref(self.ops[v]), _ptr(buf), _ptr(out),
                                     self._stream()), "tf_unpack")
        return out

    def refine(self, tol: float = 1e-10, max_outer: int = 24, inner_fraction: float = 0.25):
        """FP64 defect correction of every volume's converged field, all volumes together.

        Each outer step computes the float64 residual r = b - A c of every volume still above
        `tol` (relative 2-norm), solves the correction equation A e = r in float32 for all of them
        in shared launches (volume v runs max(100, inner_fraction * iter_v) half-sweeps, rounded
        up to an even number of launches) and adds e to c in float64. The field buffers hold e
        meanwhile; the rounded float64 result returns to field A. Metrics come from the float64
        field, which a second call continues from (solve() drops it). Per volume,
        `residual_history` lists the relative residual before every step.
        """
        lib, n = self.lib, self.n
        f64 = dict(dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            st = self._stream()
            if self._rhs is None:
                self._rhs = [torch.zeros(self.geoms[v].field_elems, dtype=torch.float32, device=self.device)
                             for v in range(n)]
                self._r2 = torch.zeros(self.csum.numel(), **f64)
                self._b2 = torch.zeros(self.csum.numel(), **f64)
                self.desc_rhs = torch.empty_like(self.desc)
                P = C.c_void_p * n
                check(lib.tf_batch_describe_rhs(n, self.geoms, self.ops, P(*[_ptr(t) for t in self.fa]),
                                                P(*[_ptr(t) for t in self.fb]), P(*[_ptr(t) for t in self.codes]),
                                                P(*[_ptr(t) for t in self._rhs]), _ptr(self.err),
                                                _ptr(self.desc_rhs)), "tf_batch_describe_rhs")
            c64 = self.c64  # a previous refinement's float64 fields, else widen the float32 ones
            if c64 is None:
                c64 = []
                for v in range(n):
                    g = self.geoms[v]
                    cur = self.fb[v] if self._final_in_b[v] else self.fa[v]
                    c = torch.empty(g.field_elems, **f64)
                    check(lib.tf_widen_f64(C.byref(g), _ptr(cur), _ptr(c), st), "tf_widen_f64")
                    c64.append(c)
            k2 = 2 * self.k
            want = [max(100, int(inner_fraction * max(r.iter, 1))) for r in self.results]
            active = np.ones(n, dtype=bool)
            hist = [[] for _ in range(n)]
            r2o = self._r2.element_size()
            for outer in range(max_outer + 1):
                for v in np.nonzero(active)[0]:
                    off = self.csum_off[v] * r2o
                    check(lib.tf_residual_f64(C.byref(self.geoms[v]), C.byref(self.ops[v]), _ptr(c64[v]),
                                              _ptr(self.codes[v]), _ptr(self._rhs[v]), _ptr(self._r2) + off,
                                              _ptr(self._b2) + off, st), "tf_residual_f64")
                r2, b2 = self._r2.cpu().numpy(), self._b2.cpu().numpy()
                for v in np.nonzero(active)[0]:
                    sl = slice(self.csum_off[v], self.csum_off[v] + self.results[v].Nx)
                    rel = math.sqrt(r2[sl].sum()) / max(math.sqrt(b2[sl].sum()), 1e-300)
                    hist[v].append(rel)
                    if rel < tol or outer == max_outer:
                        active[v] = False
                if not active.any():
                    break
                launches = [2 * (-(-want[v] // k2)) if active[v] else 0 for v in range(n)]
                for v in np.nonzero(active)[0]:
                    self.fa[v].zero_()
                self._launches = torch.tensor(launches, dtype=torch.int32).to(self.device)
                for j in range(max(launches)):
                    for cls, (w, nw) in enumerate(self._work_for([v for v in range(n) if launches[v] > j])):
                        if nw:
                            check(lib.tf_batch_advance_rhs_tile(_ptr(self.desc_rhs), _ptr(w), nw,
                                                                _ptr(self._launches), j, cls, st),
                                  "tf_batch_advance_rhs_tile")
                for v in np.nonzero(active)[0]:
                    check(lib.tf_axpy_f64(C.byref(self.geoms[v]), _ptr(c64[v]), _ptr(self.fa[v]), st), "tf_axpy_f64")
            if int(self.err.item()):
                raise _capi.TfError(int(self.err.item()), "tf_batch_advance_rhs (device)")
            for v in range(n):
                g, op = self.geoms[v], self.ops[v]
                check(lib.tf_narrow_f64(C.byref(g), C.byref(op), _ptr(c64[v]), _ptr(self.fa[v]), st), "tf_narrow_f64")
                self._final_in_b[v] = False
                check(lib.tf_layer_sums_f64(C.byref(g), C.byref(op), _ptr(c64[v]), _ptr(self.codes[v]),
                                            _ptr(self.flux) + self.flux_off[v] * 8, _ptr(self.csum) + self.csum_off[v] * 8,
                                            st), "tf_layer_sums_f64")
            flux, csum = self.flux.cpu().numpy(), self.csum.cpu().numpy()
            perc = self.perc.cpu().numpy()
            for v, res in enumerate(self.results):
                area = float(res.Ny * res.Nz)
                res.flux_1d = flux[self.flux_off[v]:self.flux_off[v] + res.Nx - 1][None] / area
                if perc[v] == 2:
                    res.flux_1d = np.zeros_like(res.flux_1d)
                c_x = csum[self.csum_off[v]:self.csum_off[v] + res.Nx][None] / area
                tau, _ = layer_metrics(res, res.flux_1d, c_x)
                res.tau = np.where(tau == 0, np.inf, tau)
                res.residual_history = hist[v]
            self.c64 = c64
        return self.results


def split_volumes(sizes, n_parts: int):
    """Whole volumes to `n_parts` devices, balanced by voxel count: largest first, each to the
    part with the fewest voxels so far (ties to the lower part). Returns one sorted index list
    per part; every index appears exactly once. The volumes are independent, so no part ever
    waits for another (the natural shard of a batch of volumes)."""
    if n_parts < 1:
        raise ValueError("n_parts must be >= 1")
    load = [0] * n_parts
    parts = [[] for _ in range(n_parts)]
    for i in sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i)):
        p = min(range(n_parts), key=lambda j: (load[j], j))
        parts[p].append(i)
        load[p] += int(sizes[i])
    return [sorted(p) for p in parts]


class MultiDeviceBatchSolve:
    """BatchSolve over several GPUs of one process: whole volumes per device (split_volumes),
    one BatchSolve per entry of `devices`, one host thread per distinct device (the parts of a
    device listed twice run in turn); results come back in the caller's order. No data crosses
    devices (each volume lives on one GPU)."""

    def __init__(self, volumes, devices, periodic=False, omega=None):
        vols = [np.asarray(v) for v in volumes]
        n = len(vols)
        per = list(periodic) if isinstance(periodic, (list, tuple, np.ndarray)) else [bool(periodic)] * n
        om = list(omega) if isinstance(omega, (list, tuple, np.ndarray)) else [omega] * n
        if len(per) != n or len(om) != n:
            raise ValueError("periodic / omega must give one entry per volume")
        self.devices = [torch.device(d) for d in devices]
        self.parts = split_volumes([v.size for v in vols], len(self.devices))
        self.batches = [BatchSolve([vols[i] for i in p], periodic=[per[i] for i in p], omega=[om[i] for i in p],
                                   device=d) if p else None for p, d in zip(self.parts, self.devices)]
        self.n = n

    def solve(self, **kwargs):
        errors = []
        by_device = {}
        for b in self.batches:
            if b is not None:
                by_device.setdefault(str(b.device), []).append(b)

        def run(batches):
            try:
                for b in batches:
                    with torch.cuda.device(b.device):
                        b.solve(**kwargs)
            except BaseException as e:  # re-raised on the calling thread
                errors.append(e)

        threads = [threading.Thread(target=run, args=(bs,)) for bs in by_device.values()]
        start = timer()
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        self.walltime = timer() - start
        if errors:
            raise errors[0]
        return self.results

    @property
    def results(self):
        out = [None] * self.n
        for p, b in zip(self.parts, self.batches):
            if b is not None:
                for j, i in enumerate(p):
                    out[i] = b.results[j]
        return out
