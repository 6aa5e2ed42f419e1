"""Helpers shared by the GPU tests: move math-layout numpy blocks into the
library's column-major tensors and back."""
import numpy as np


def upload(data, A, B, d):
    """A (N,n,n), B (N-1,n,n), d (N,n,k) math blocks -> data.*_tensor[:, :, :N]."""
    import torch
    N = A.shape[0]
    dt = data.dtype
    dev = data.A_tensor.device
    data.A_tensor[:, :, :N] = torch.from_numpy(np.ascontiguousarray(A)).to(dev, dt).permute(1, 2, 0)
    if N > 1:
        data.B_tensor[:, :, :N - 1] = torch.from_numpy(np.ascontiguousarray(B)).to(dev, dt).permute(1, 2, 0)
    data.d_tensor[:, :, :N] = torch.from_numpy(np.ascontiguousarray(d)).to(dev, dt).permute(1, 2, 0)


def download_x(data, N=None):
    """data.d_tensor[:, :, :N] -> (N, n, k) float64 numpy."""
    N = data.N if N is None else N
    return data.d_tensor[:, :, :N].permute(2, 0, 1).double().cpu().numpy()


def download_blocks(t, count):
    """column-major (n, n, count) tensor view -> (count, n, n) numpy math blocks."""
    return t[:, :, :count].permute(2, 0, 1).double().cpu().numpy()
