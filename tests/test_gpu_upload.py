"""Host upload and download (bss_upload / bss_download): the whole-block
copy, and the upper-triangle upload whose A_i are defined by their upper
triangles alone, as the reference's potrf(FILL_MODE_UPPER) reads them
(src/backbone_cuda.jl:21-33, 77-99), mirrored on the device.  The lower
triangles of the host A_i hold junk, so a solution that matches the oracle
on the symmetrized upper triangle shows the junk never reached a kernel."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_blocks

pytestmark = pytest.mark.gpu


def _host(X, torch_dtype):
    """math blocks (count, a, b) -> pinned host tensor in the column-major block layout (count, b, a)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.swapaxes(X, 1, 2))).to(torch_dtype).pin_memory()


def _junk_lower(A, rng):
    J = A.copy()
    il = np.tril_indices(A.shape[1], -1)
    J[:, il[0], il[1]] = rng.standard_normal((A.shape[0], len(il[0]))) * 1e3
    return J


def _sym_upper(A):
    U = np.triu(A)
    return U + np.swapaxes(np.triu(A, 1), 1, 2)


@pytest.mark.parametrize("n,T", [(64, "f64"), (128, "f64"), (16, "f64"), (48, "f64"), (33, "f64"),
                                 (96, "f32"), (128, "f32"), (64, "f32")])
def test_upload_upper_mirrors_and_solves(n, T):
    import torch
    import blockstructuredsolvers_gb300 as bss
    tdt = torch.float64 if T == "f64" else torch.float32
    es = 8 if T == "f64" else 4
    rng = np.random.default_rng(4100 + n + es)
    N, k = 300, 2
    A, B, d = O.gen_shifted_family(rng, N, n, k)
    A = A.astype(np.float32).astype(np.float64) if T == "f32" else A
    B = B.astype(np.float32).astype(np.float64) if T == "f32" else B
    d = d.astype(np.float32).astype(np.float64) if T == "f32" else d
    Aj = _junk_lower(A, rng)
    data = bss.initialize_batched(N, n, tdt, k=k)
    padA = download_blocks(data.A_tensor[:, :, N:], data.N - N) if data.N > N else None
    moved = bss.upload(data, _host(Aj, tdt), _host(B, tdt), _host(d, tdt), upper=True)
    assert moved == es * (N * n * n + (N - 1) * n * n + N * n * k)
    bss.synchronize(data)
    S = _sym_upper(Aj)
    assert np.array_equal(download_blocks(data.A_tensor, N), S)
    if padA is not None:  # padding blocks untouched
        assert np.array_equal(download_blocks(data.A_tensor[:, :, N:], data.N - N), padA)
    bss.factorize_(data)
    bss.solve_(data)
    x = torch.empty((N, k, n), dtype=tdt).pin_memory()
    bss.download(data, x)
    bss.synchronize(data)
    xm = x.double().numpy().transpose(0, 2, 1)
    x_ref = O.cpu_solve(S, B, d)
    assert O.rel_error(xm, x_ref) <= (1e-4 if T == "f32" else 1e-10)


def test_upload_full_copies_bytes():
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(4200)
    N, n, k = 77, 64, 3
    A, B, d = O.gen_shifted_family(rng, N, n, k)
    Aj = _junk_lower(A, rng)
    data = bss.initialize_batched(N, n, torch.float64, k=k)
    moved = bss.upload(data, _host(Aj, torch.float64), _host(B, torch.float64), _host(d, torch.float64))
    assert moved == 8 * (N * n * n + (N - 1) * n * n + N * n * k)
    bss.synchronize(data)
    assert np.array_equal(download_blocks(data.A_tensor, N), Aj)
    assert np.array_equal(download_blocks(data.B_tensor, N - 1), B)
    assert np.array_equal(data.d_tensor[:, :, :N].permute(2, 0, 1).cpu().numpy(), d)


def test_upload_mixed_headline_shape_and_numpy_layouts():
    """Mixed precision at the headline block size n = 64, numpy host arrays in
    both accepted layouts (row-major (N, n, n) and column-major (n, n, N))."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(4300)
    N, n = 1500, 64
    A, B, d = O.gen_shifted_family(rng, N, n, 1)
    Aj = _junk_lower(A, rng)
    data = bss.initialize_batched(N, n, torch.float64, k=1, precision="mixed")
    Ah = np.ascontiguousarray(np.swapaxes(Aj, 1, 2))        # (N, c, r) row-major
    Bh = np.asfortranarray(np.transpose(B, (1, 2, 0)))      # (r, c, N) column-major
    dh = np.ascontiguousarray(np.swapaxes(d, 1, 2))
    bss.upload(data, Ah, Bh, dh, upper=True)
    bss.factorize_(data)
    bss.solve_(data)
    x = np.empty((N, 1, n))
    bss.download(data, x)
    bss.synchronize(data)
    S = _sym_upper(Aj)
    xm = x.transpose(0, 2, 1)
    info = bss.get_info(data)
    assert info["rel_residual"] <= 1e-12
    assert O.rel_residual(S, B, xm, d) <= 1e-12
    assert O.rel_error(xm, O.cpu_solve(S, B, d)) <= 1e-10


def test_upload_seq_handle_and_partial():
    """The sequential solver's handle; uploads of d alone keep A and B."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(4400)
    N, n = 40, 64
    A, B, d = O.gen_shifted_family(rng, N, n, 1)
    data = bss.initialize_seq(N, n, torch.float64)
    bss.upload(data, _host(_junk_lower(A, rng), torch.float64), _host(B, torch.float64), _host(d, torch.float64),
               upper=True)
    bss.factorize_(data)
    bss.solve_(data)
    x1 = np.empty((N, 1, n))
    bss.download(data, x1)
    bss.synchronize(data)
    assert O.rel_error(x1.transpose(0, 2, 1), O.cpu_solve(A, B, d)) <= 1e-10
    d2 = rng.random((N, n, 1))
    assert bss.upload(data, d=_host(d2, torch.float64)) == 8 * N * n
    bss.solve_(data)
    x2 = np.empty((N, 1, n))
    bss.download(data, x2)
    bss.synchronize(data)
    assert O.rel_error(x2.transpose(0, 2, 1), O.cpu_solve(A, B, d2)) <= 1e-10


def test_upload_rejects_bad_arrays():
    import torch
    import blockstructuredsolvers_gb300 as bss
    data = bss.initialize_batched(10, 16, torch.float64)
    with pytest.raises(ValueError):
        bss.upload(data, np.zeros((10, 16, 15)))                 # wrong shape
    with pytest.raises(ValueError):
        bss.upload(data, np.zeros((10, 16, 16), np.float32))     # wrong dtype
    with pytest.raises(ValueError):
        bss.upload(data, np.zeros((16, 16, 10)))                 # (n, n, N) but row-major
    with pytest.raises(ValueError):
        bss.upload(data, torch.zeros((10, 16, 16), dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        x = np.zeros((10, 1, 16))
        x.flags.writeable = False
        bss.download(data, x)
    from blockstructuredsolvers_gb300 import _lib
    with pytest.raises(bss.BSSError):
        _lib.check(_lib.load().bss_upload(data.handle, None, None, None, 7, None))
