"""Host-array checks of the upload / download API (blockstructuredsolvers_gb300
.upload / .download): which numpy arrays and CPU torch tensors are accepted as
column-major blocks, and that the address handed to the C ABI is the array's
own memory (nothing copied).  Host logic only: no GPU."""
import numpy as np
import pytest


def _check(X, dims, dtype, **kw):
    import blockstructuredsolvers_gb300 as bss
    return bss._host_blocks(X, dims, dtype, "X", **kw)


def test_accepts_both_layouts_without_copies():
    import torch
    n, k, N = 6, 3, 5
    row = np.zeros((N, k, n))                        # (count, b, a) row-major
    col = np.asfortranarray(np.zeros((n, k, N)))     # (a, b, count) column-major
    assert _check(row, (n, k, N), torch.float64) == row.ctypes.data
    assert _check(col, (n, k, N), torch.float64) == col.ctypes.data
    t = torch.zeros((N, k, n), dtype=torch.float32)
    assert _check(t, (n, k, N), torch.float32) == t.data_ptr()
    tc = torch.zeros((N, k, n), dtype=torch.float64).permute(2, 1, 0)  # (n, k, N), strides (1, n, n k)
    assert tuple(tc.stride()) == (1, n, n * k)
    assert _check(tc, (n, k, N), torch.float64) == tc.data_ptr()


@pytest.mark.parametrize("bad", ["shape", "dtype", "order", "strided", "list"])
def test_rejects(bad):
    import torch
    n, N = 4, 7
    X = {"shape": np.zeros((N, n, n + 1)),
         "dtype": np.zeros((N, n, n), np.float32),
         "order": np.zeros((n, n, N)),                          # (a, b, count) but row-major
         "strided": np.zeros((N, n, 2 * n))[:, :, ::2],         # right shape, not dense
         "list": [[0.0] * n] * n}[bad]
    with pytest.raises(ValueError):
        _check(X, (n, n, N), torch.float64)


def test_rejects_read_only_output_and_device_tensors():
    import torch
    x = np.zeros((3, 1, 4))
    x.flags.writeable = False
    with pytest.raises(ValueError):
        _check(x, (4, 1, 3), torch.float64, writable=True)
    assert _check(x, (4, 1, 3), torch.float64) == x.ctypes.data  # fine as an input
    if torch.cuda.is_available():
        with pytest.raises(ValueError):
            _check(torch.zeros((3, 1, 4), dtype=torch.float64, device="cuda"), (4, 1, 3), torch.float64)


def test_upload_constants_match_header():
    import os
    import re
    from blockstructuredsolvers_gb300 import _lib
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "bss.h")).read()
    for name in ("BSS_UPLOAD_FULL", "BSS_UPLOAD_UPPER"):
        m = re.search(r"#define\s+%s\s+(\d+)" % name, hdr)
        assert m and int(m.group(1)) == getattr(_lib, name)
