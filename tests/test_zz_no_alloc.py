"""GPU test of tf_batch_converge_static, the allocation-free convergence step.

Callers that cannot give the library device memory beyond their own buffers (for example a
host whose GPU memory another framework's pool has reserved, or a binding without the CUDA
allocator) use this entry point; it keeps the per-plane sums in a static array inside the
library. Here it must decide exactly like the arena-based pair tf_batch_layer_sums +
tf_batch_check on the same fields, on two consecutive calls (the static array keeps the first
call's contents when the second one starts). Collected last on purpose (file name).
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _state(d):
    from taufactor_gb300._capi import TfBatchState

    return TfBatchState(*(d[k].data_ptr() for k in ("status", "perc", "conv_iter", "conv_parity", "old_tau", "tau",
                                                     "rel", "d_rel", "iter_base")))


def _fresh_state(b):
    keys = ("status", "perc", "conv_iter", "conv_parity", "old_tau", "tau", "rel", "d_rel", "iter_base")
    return {k: getattr(b, k).clone() for k in keys}


def test_static_scratch_converge_matches_arena_path():
    import taufactor_gb300 as tg
    from taufactor_gb300._capi import TF_ERR_ARG, TF_ERR_UNSUPPORTED, check
    from taufactor_gb300.synthetic import blurred_noise

    shapes = [(32, 48, 64), (40, 32, 96), (24, 40, 128)]  # tile classes 0, 2, 1
    vols = [blurred_noise(s, 2.0, 0.55, 300 + i) for i, s in enumerate(shapes)]
    b = tg.BatchSolve(vols, periodic=[False, True, False])
    lib, st = b.lib, b._stream()
    flux_len, csum_len = b.flux.numel(), b.csum.numel()
    arena_state, static_state = _fresh_state(b), _fresh_state(b)
    parity = 0
    for call in range(2):
        for _ in range(25):  # 100 half-sweeps of every volume
            for cls, (w, nw) in enumerate(b.works):
                if nw:
                    check(lib.tf_batch_advance_tile(b.desc.data_ptr(), w.data_ptr(), nw, b.status.data_ptr(),
                                                    parity, cls, st), "tf_batch_advance_tile")
            parity ^= 1
        # the existing path: sums into caller arenas, then the decision
        check(lib.tf_batch_layer_sums(b.desc.data_ptr(), b.planes.data_ptr(), b.n_planes, b.status.data_ptr(),
                                      parity, b.flux.data_ptr(), b.csum.data_ptr(), st), "tf_batch_layer_sums")
        check(lib.tf_batch_check(b.desc.data_ptr(), b.n, b.flux.data_ptr(), _state(arena_state), 1e-9, call,
                                 parity, st), "tf_batch_check")
        # the allocation-free path on the same fields
        n0 = lib.tf_launch_count()
        check(lib.tf_batch_converge_static(b.desc.data_ptr(), b.planes.data_ptr(), b.n_planes, b.n, flux_len,
                                           csum_len, _state(static_state), 1e-9, call, parity, st),
              "tf_batch_converge_static")
        assert lib.tf_launch_count() - n0 == 2
        torch.cuda.synchronize()
        # the same kernels on the same fields: the decisions and the float64 metrics agree bit for bit
        for k in ("status", "conv_iter", "conv_parity", "tau", "rel", "d_rel", "old_tau"):
            assert torch.equal(arena_state[k], static_state[k]), (call, k)
        assert np.all(np.isfinite(static_state["tau"].cpu().numpy()))
    # sizes beyond the static capacity are refused before anything is launched
    n0 = lib.tf_launch_count()
    rc = lib.tf_batch_converge_static(b.desc.data_ptr(), b.planes.data_ptr(), b.n_planes, b.n, 65537, csum_len,
                                      _state(static_state), 1e-9, 0, parity, st)
    assert rc == TF_ERR_UNSUPPORTED
    # arguments that disagree with what tf_batch_describe built are refused too: arena lengths
    # shorter than the descriptor's offsets need, more volumes than it holds, a table it never built
    for args in ((b.desc.data_ptr(), b.n, flux_len - 1, csum_len), (b.desc.data_ptr(), b.n, flux_len, csum_len - 1),
                 (b.desc.data_ptr(), b.n + 1, flux_len, csum_len), (b.desc.data_ptr() + 64, b.n, flux_len, csum_len)):
        desc, n_vol, fl, cl = args
        rc = lib.tf_batch_converge_static(desc, b.planes.data_ptr(), b.n_planes, n_vol, fl, cl, _state(static_state),
                                          1e-9, 0, parity, st)
        assert rc == TF_ERR_ARG, args
    assert lib.tf_launch_count() == n0
