"""GPU tests of the request server (bss_server_*) and the device Kalman
block builder (bss_kf_build), against the oracle.

Tolerances: the device-built Kalman blocks match the host restatement of
build_kf_blocks to 1e-13 relative (same formulas, different summation
order); mixed-precision results reach relative residual <= 1e-12 and
relative error <= 1e-9 vs the CPU block Cholesky oracle; plain FP64 results
relative error <= 1e-10.  A request's result is bitwise identical served
alone and in a concurrent mix.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bss():
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    assert torch.cuda.is_available()
    _lib.load()
    return bss


def _pinned(shape):
    import torch
    return torch.zeros(shape, dtype=torch.float64).pin_memory()


def _st(M):
    """math blocks (N, r, c) -> storage order (N, c, r) contiguous (column-major blocks)."""
    return np.ascontiguousarray(np.swapaxes(M, 1, 2))


def _x(t):
    """storage (N, k, n) -> math (N, n, k)."""
    return np.swapaxes(t.numpy(), 1, 2)


def _systems(seed, shapes):
    rng = np.random.default_rng(seed)
    out = []
    for (N, n, k) in shapes:
        A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=2.0 * max(n, 6), b_scale=0.5)
        out.append((A, B, d))
    return out


SHAPES = [(50, 8, 1), (300, 16, 2), (1200, 32, 1), (77, 64, 3), (500, 48, 1), (2, 16, 1), (1, 24, 2), (90, 96, 1)]


def _submit_all(srv, probs, keep=False):
    reqs = []
    for (A, B, d) in probs:
        N, n, _ = A.shape
        k = d.shape[2]
        x = _pinned((N, k, n))
        rid, fid = srv.submit(_st(A), _st(B) if N > 1 else None, _st(d), x, keep=keep)
        reqs.append((rid, fid, x))
    return reqs


def test_server_mixed_systems(bss):
    probs = _systems(1, SHAPES)
    srv = bss.Server(streams=4)
    reqs = _submit_all(srv, probs)
    for (rid, _, x), (A, B, d) in zip(reqs, probs):
        info = srv.wait(rid)
        xs = _x(x)
        assert info["rel_residual"] <= 1e-12
        assert O.rel_residual(A, B, xs, d) <= 1e-12
        assert O.rel_error(xs, O.cpu_solve(A, B, d)) <= 1e-9
    st = srv.stats()
    assert st["completed"] == len(probs) and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()


def test_server_plain_fp64(bss):
    probs = _systems(2, SHAPES[:5])
    srv = bss.Server(precision="plain")
    reqs = _submit_all(srv, probs)
    for (rid, _, x), (A, B, d) in zip(reqs, probs):
        srv.wait(rid)
        assert O.rel_error(_x(x), O.cpu_solve(A, B, d)) <= 1e-10
    srv.close()


def test_server_same_result_alone_and_in_mix(bss):
    """Each request alone in a fresh server and inside a concurrent mix of
    many requests on several streams: bitwise the same solution."""
    probs = _systems(3, SHAPES * 3)
    srv = bss.Server(streams=8)
    mix = _submit_all(srv, probs)
    for rid, _, _ in mix:
        srv.wait(rid)
    srv.close()
    for i in (0, 2, 3, 7, 9, 20):
        alone = bss.Server(streams=1)
        (rid, _, x), = _submit_all(alone, [probs[i]])
        alone.wait(rid)
        assert np.array_equal(x.numpy(), mix[i][2].numpy())
        alone.close()


def test_server_repeat_rhs_on_resident_factor(bss):
    probs = _systems(4, SHAPES[:4])
    srv = bss.Server()
    reqs = _submit_all(srv, probs, keep=True)
    rng = np.random.default_rng(44)
    rhs = []
    for (rid, fid, _), (A, B, d) in zip(reqs, probs):
        assert fid == rid
        d2 = rng.standard_normal(d.shape)
        x2 = _pinned((A.shape[0], d.shape[2], A.shape[1]))
        d2s = _st(d2)
        rhs.append((srv.submit_rhs(fid, d2s, x2), x2, d2, d2s))
    for (rid, _, _), (A, B, d) in zip(reqs, probs):
        srv.wait(rid)
    for (rid2, x2, d2, _), (A, B, d) in zip(rhs, probs):
        info = srv.wait(rid2)
        assert O.rel_residual(A, B, _x(x2), d2) <= 1e-12
    assert srv.stats()["resident_factors"] == len(probs)
    for (_, fid, _) in reqs:
        srv.release(fid)
    assert srv.stats()["resident_factors"] == 0
    srv.close()


def test_server_budget_evicts_and_rejects(bss):
    """A budget that holds about two of these factors: later keeps evict the
    least recently used idle factor; an RHS on it then fails; a request
    larger than the whole budget fails with BSS_ERR_OOM."""
    from blockstructuredsolvers_gb300 import _lib
    probs = _systems(5, [(400, 64, 1)] * 4)
    srv = bss.Server(hbm_budget_bytes=2 * 400 * 64 * 64 * 8 * 4)
    reqs = []
    for p in probs:  # one at a time, so the eviction order is defined
        (r,) = _submit_all(srv, [p], keep=True)
        srv.wait(r[0])
        reqs.append(r)
    st = srv.stats()
    assert st["evictions"] >= 1
    x = _pinned((400, 1, 64))
    with pytest.raises(bss.BSSError) as ei:
        srv.submit_rhs(reqs[0][1], _st(probs[0][2]), x)
    assert ei.value.code == _lib.BSS_ERR_STATE
    rid = srv.submit_rhs(reqs[3][1], _st(probs[3][2]), x)  # the most recent one is resident
    srv.wait(rid)
    big = _systems(6, [(6000, 64, 1)])
    (r,) = _submit_all(srv, big)
    info = srv.wait(r[0], check=False)
    assert info["status"] == _lib.BSS_ERR_OOM
    srv.close()


def test_kf_build_matches_host_restatement(bss):
    import torch
    rng = np.random.default_rng(7)
    for (N, n, k, boundary) in [(40, 16, 1, False), (33, 12, 2, True), (5, 64, 1, True)]:
        F, H, Qinv, Rinv, Y = O.gen_kalman_model(rng, N, n, k)
        m = H.shape[0]
        P0inv = np.eye(n) * 0.7 if boundary else None
        x0 = rng.standard_normal(n) if boundary else None
        A, B, d = O.kf_blocks(F, H, Qinv, Rinv, Y, P0inv, x0)
        cm = lambda M: torch.from_numpy(np.asfortranarray(M)).cuda().T.contiguous().T  # column-major device
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        Fd, Hd, Qd, Rd = cm(F), cm(H), cm(Qinv), cm(Rinv)
        Yd = dev(np.swapaxes(Y, 1, 2)).permute(2, 1, 0)  # (m, k, N) column-major
        Ad = bss.colmajor_empty((n, n, N), torch.float64)
        Bd = bss.colmajor_empty((n, n, max(N - 1, 1)), torch.float64)
        dd = bss.colmajor_empty((n, k, N), torch.float64)
        bss.kf_build(Fd, Hd, Qd, Rd, Yd, Ad, Bd, dd, P0inv=cm(P0inv) if boundary else None,
                     x0=dev(x0) if boundary else None)
        torch.cuda.synchronize()
        Ag = Ad.permute(2, 0, 1).cpu().numpy()
        Bg = Bd.permute(2, 0, 1).cpu().numpy()[: N - 1]
        dg = dd.permute(2, 0, 1).cpu().numpy()
        assert np.abs(Ag - A).max() <= 1e-13 * np.abs(A).max()
        assert np.abs(Bg - B).max() <= 1e-13 * np.abs(B).max()
        assert np.abs(dg - d).max() <= 1e-13 * np.abs(d).max()
        assert np.array_equal(Ag, np.swapaxes(Ag, 1, 2))


def test_server_kalman_requests_and_repeat_rhs(bss):
    rng = np.random.default_rng(8)
    srv = bss.Server()
    cases = []
    for (N, n) in [(300, 8), (1000, 16), (150, 32), (64, 64)]:
        F, H, Qinv, Rinv, Y = O.gen_kalman_model(rng, N, n, 1)
        x = _pinned((N, 1, n))
        fm = lambda M: np.ascontiguousarray(M.T)  # column-major
        Ys = np.ascontiguousarray(np.swapaxes(Y, 1, 2))  # (N, k, m)
        rid, fid = srv.submit_kalman(fm(F), fm(H), fm(Qinv), fm(Rinv), Ys, x, keep=True)
        cases.append((rid, fid, x, (F, H, Qinv, Rinv, Y)))
    for rid, fid, x, (F, H, Qinv, Rinv, Y) in cases:
        info = srv.wait(rid)
        A, B, d = O.kf_blocks(F, H, Qinv, Rinv, Y)
        assert O.rel_residual(A, B, _x(x), d) <= 1e-12
        assert O.rel_error(_x(x), O.cpu_solve(A, B, d)) <= 1e-9
        # repeat right-hand side: new observations on the resident factor
        Y2 = rng.standard_normal(Y.shape)
        x2 = _pinned(tuple(x.shape))
        Y2s = np.ascontiguousarray(np.swapaxes(Y2, 1, 2))
        r2 = srv.submit_rhs(fid, Y2s, x2)
        srv.wait(r2)
        A, B, d2 = O.kf_blocks(F, H, Qinv, Rinv, Y2)
        assert O.rel_residual(A, B, _x(x2), d2) <= 1e-12
    srv.close()
