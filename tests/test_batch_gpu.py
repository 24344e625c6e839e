"""GPU tests of the uneven-shape batched solve: every volume's result equals the drop-in
single-volume solver's (same half-sweeps bit for bit, same device layer sums, same convergence
rule), with and without CUDA-graph capture."""
import numpy as np
import pytest

from cases import random_binary

pytestmark = pytest.mark.gpu

import taufactor_gb300 as tg  # noqa: E402
from taufactor_gb300.synthetic import blurred_noise  # noqa: E402

SHAPES = [(32, 48, 64), (40, 32, 96), (48, 64, 32), (24, 40, 72), (64, 32, 48), (36, 48, 40)]


def _volumes():
    vols = [blurred_noise(s, 2.0, 0.55, 100 + i) for i, s in enumerate(SHAPES)]
    periodic = [i % 2 == 1 for i in range(len(vols))]
    return vols, periodic


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_single_volume_solvers(graph):
    vols, periodic = _volumes()
    b = tg.BatchSolve(vols, periodic=periodic)
    res = b.solve(conv_crit=1e-3, graph=graph)
    for v, (img, per) in enumerate(zip(vols, periodic)):
        s = (tg.PeriodicSolver if per else tg.Solver)(img)
        s.solve(verbose=False, conv_crit=1e-3)
        assert res[v].converged and s.converged
        assert res[v].iter == s.iter, (v, res[v].iter, s.iter)
        np.testing.assert_allclose(res[v].D_eff, s.D_eff, rtol=1e-12)
        np.testing.assert_allclose(res[v].tau, s.tau, rtol=1e-12)
        np.testing.assert_allclose(res[v].tau_x, s.tau_x, rtol=1e-9, atol=1e-12)
        got = b.field(v).cpu().numpy()[:, :, 1:-1, 1:-1]
        want = s.field.cpu().numpy()[:, :, 1:-1, 1:-1]
        assert np.array_equal(got, want), v


def test_batch_x_chunks_match_single_volume_solvers(monkeypatch):
    """Work items that cover tile columns in several x-chunks (20 planes each here) give the
    single-volume results bit for bit, also with the FP64 correction."""
    import taufactor_gb300.batch as batch_mod

    monkeypatch.setattr(batch_mod, "CHUNK", 20)
    vols, periodic = _volumes()
    b = tg.BatchSolve(vols, periodic=periodic)
    assert b.n_work > sum(b._tiles)  # more work items than tile columns: columns are chunked
    res = b.solve(conv_crit=1e-3)
    for v, (img, per) in enumerate(zip(vols, periodic)):
        s = (tg.PeriodicSolver if per else tg.Solver)(img)
        s.solve(verbose=False, conv_crit=1e-3)
        assert res[v].iter == s.iter
        np.testing.assert_allclose(res[v].D_eff, s.D_eff, rtol=1e-12)
        assert np.array_equal(b.field(v).cpu().numpy()[:, :, 1:-1, 1:-1], s.field.cpu().numpy()[:, :, 1:-1, 1:-1])
    res = b.refine(tol=1e-10)
    assert all(r.residual_history[-1] < 1e-10 for r in res)


def test_batch_short_chunks_and_compaction_match_single_volume_solvers(monkeypatch):
    """Chunks shorter than the fused depth (down to 1 plane) and work lists compacted as volumes
    converge give the single-volume results bit for bit."""
    import taufactor_gb300.batch as batch_mod

    monkeypatch.setattr(batch_mod, "CHUNK", 6)
    monkeypatch.setattr(batch_mod, "MIN_CHUNK", 1)
    vols, periodic = _volumes()
    b = tg.BatchSolve(vols, periodic=periodic)
    n0 = b.n_work
    res = b.solve(conv_crit=1e-3, poll=1)
    assert len(b._work_cache) > 1 and b.n_work < n0  # the list shrank as volumes converged
    for v, (img, per) in enumerate(zip(vols, periodic)):
        s = (tg.PeriodicSolver if per else tg.Solver)(img)
        s.solve(verbose=False, conv_crit=1e-3)
        assert res[v].iter == s.iter
        np.testing.assert_allclose(res[v].D_eff, s.D_eff, rtol=1e-12)
        assert np.array_equal(b.field(v).cpu().numpy()[:, :, 1:-1, 1:-1], s.field.cpu().numpy()[:, :, 1:-1, 1:-1])
    res = b.refine(tol=1e-10)
    assert all(r.residual_history[-1] < 1e-10 for r in res)


def test_batch_tile_classes_match_single_volume_solvers():
    """Volumes on 16 x 128 tiles (z-extent a multiple of 128) and on 32 x 64 tiles (y-extent a
    multiple of 32), each class swept on its own stream next to the volumes on 16 x 64 tiles,
    give the single-volume results bit for bit, with and without the graph, and through the
    FP64 correction."""
    shapes = [(32, 32, 128), (24, 48, 64), (28, 16, 256), (36, 64, 96), (20, 32, 72), (30, 40, 96)]
    vols = [blurred_noise(s, 2.0, 0.55, 400 + i) for i, s in enumerate(shapes)]
    periodic = [i % 2 == 1 for i in range(len(vols))]
    for graph in (True, False):
        b = tg.BatchSolve(vols, periodic=periodic)
        assert [b.ops[v].tile for v in range(len(vols))] == [1, 0, 1, 2, 2, 0]
        assert all(nw > 0 for _, nw in b.works)
        res = b.solve(conv_crit=1e-3, graph=graph)
        for v, (img, per) in enumerate(zip(vols, periodic)):
            s = (tg.PeriodicSolver if per else tg.Solver)(img)
            s.solve(verbose=False, conv_crit=1e-3)
            assert res[v].iter == s.iter, (v, res[v].iter, s.iter)
            np.testing.assert_allclose(res[v].D_eff, s.D_eff, rtol=1e-12)
            assert np.array_equal(b.field(v).cpu().numpy()[:, :, 1:-1, 1:-1],
                                  s.field.cpu().numpy()[:, :, 1:-1, 1:-1]), v
    res = b.refine(tol=1e-10)
    assert all(r.residual_history[-1] < 1e-10 for r in res)


def test_batch_non_percolating_volume():
    vols, periodic = _volumes()
    dead = np.zeros((20, 16, 32), dtype=np.uint8)
    dead[:5] = 1  # touches the inlet only
    b = tg.BatchSolve(vols[:2] + [dead], periodic=periodic[:2] + [False])
    res = b.solve(conv_crit=1e-3)
    assert res[2].converged and np.isinf(res[2].tau).all()
    assert np.all(res[2].D_eff == 0)
    assert all(r.converged for r in res)


def test_batch_refine_matches_single_volume_refine():
    vols, periodic = _volumes()
    b = tg.BatchSolve(vols[:3], periodic=periodic[:3])
    res = b.solve(conv_crit=1e-3, refine={"tol": 1e-11})
    for v in range(3):
        s = (tg.PeriodicSolver if periodic[v] else tg.Solver)(vols[v])
        s.solve(verbose=False, conv_crit=1e-3, refine={"tol": 1e-11})
        assert res[v].residual_history[-1] < 1e-11
        np.testing.assert_allclose(res[v].D_eff, s.D_eff, rtol=1e-10)


def test_batch_rejects_bad_input():
    with pytest.raises(ValueError):
        tg.BatchSolve([np.full((8, 8, 8), 3)])
    with pytest.raises(tg.solvers._capi.TfError):
        tg.BatchSolve([random_binary((9, 9, 9), 1)], periodic=True)


def test_batch_refine_with_dead_volume_and_repeat():
    vols, periodic = _volumes()
    dead = np.zeros((32, 32, 32), dtype=np.uint8)
    dead[:20] = 1  # touches the inlet only: no spanning path
    b = tg.BatchSolve(vols[:2] + [dead], periodic=periodic[:2] + [False])
    res = b.solve(conv_crit=1e-3, refine={"tol": 1e-10})
    assert np.all(res[2].D_eff == 0) and np.isinf(res[2].tau).all()
    d1 = [r.D_eff.copy() for r in res[:2]]
    assert all(r.residual_history[-1] < 1e-10 for r in res[:2])
    res = b.refine(tol=1e-12)  # refining again starts from the refined field
    for r, d in zip(res[:2], d1):
        assert r.residual_history[0] < 1e-10 and r.residual_history[-1] < 1e-12
        np.testing.assert_allclose(r.D_eff, d, rtol=1e-9)


def test_device_split_equals_one_batch():
    """MultiDeviceBatchSolve: whole volumes per device, one host thread each (here two parts on
    the same GPU: independent batches that never wait on each other); every volume's result equals
    the single batch's, in the caller's order."""
    from taufactor_gb300.synthetic import blurred_noise

    shapes = [(32, 48, 64), (40, 32, 96), (24, 40, 128), (48, 48, 32), (32, 64, 64)]
    vols = [blurred_noise(s, 2.0, 0.55, 500 + i) for i, s in enumerate(shapes)]
    per = [i % 2 == 1 for i in range(len(vols))]
    one = tg.BatchSolve(vols, periodic=per).solve(conv_crit=1e-3)
    m = tg.MultiDeviceBatchSolve(vols, devices=["cuda:0", "cuda:0"], periodic=per)
    assert sorted(i for p in m.parts for i in p) == list(range(len(vols))) and all(m.parts)
    split = m.solve(conv_crit=1e-3)
    for a, b in zip(one, split):
        assert a.iter == b.iter
        assert np.array_equal(a.D_eff, b.D_eff) and np.array_equal(a.tau, b.tau)


def test_batch_matches_the_oracle_directly():
    """The batched solve against the oracle itself (not through the single-volume solver):
    the reference's iteration count and D_eff (float32 sweeps, float64 layer means), binary and
    periodic volumes of three shapes in one batch."""
    from oracle.sor import OracleSolve

    shapes = [(20, 16, 24), (16, 24, 20), (24, 20, 16)]
    vols = [blurred_noise(s, 1.5, 0.6, 300 + i) for i, s in enumerate(shapes)]
    periodic = [False, True, False]
    res = tg.BatchSolve(vols, periodic=periodic).solve(conv_crit=1e-3)
    for v, (img, per) in enumerate(zip(vols, periodic)):
        o = OracleSolve(img, kind="periodic" if per else "binary")
        o.solve(conv_crit=1e-3)
        assert res[v].iter == o.iter, (v, res[v].iter, o.iter)
        np.testing.assert_allclose(res[v].D_eff, o.D_eff, rtol=1e-6)
