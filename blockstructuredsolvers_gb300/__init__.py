"""GB300 (sm_103a) batched block-tridiagonal SPD solver.

Python mirror of BlockStructuredSolvers.jl's GPU API (src/BlockStructuredSolvers.jl:9-11
exports) over the C ABI of ``libbss_gb300.so`` (``include/bss.h``):

    data = initialize_batched(N, n, torch.float64)   # initialize_batched(N, n, T, CuArray)
    data.A_tensor.copy_(A); data.B_tensor.copy_(B); data.d_tensor.copy_(d)
    factorize_(data)                                  # factorize!(data)
    solve_(data)                                      # solve!(data): d_tensor <- x

``A_tensor`` (n x n x N), ``B_tensor`` (n x n x (N-1)) and ``d_tensor``
(n x k x N) are torch views of library-owned device memory with Julia's
column-major strides, so ``data.A_tensor[:, :, i]`` is the block A_i exactly
as ``data.A_tensor[:, :, i]`` is in Julia, and ``A_list[i]`` aliases it.

All compute runs in the sm_103a kernels of the library; there is no CPU or
PyTorch fallback.  Loading fails loudly if the library is missing.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import BSSError, NotSPDError  # noqa: F401

__all__ = [
    "BlockTriDiagData_batched", "BlockTriDiagData_seq", "initialize_batched", "initialize_seq",
    "factorize_", "solve_", "factorize", "solve", "synchronize", "upload", "download", "get_info", "residual",
    "plan_reference", "BSSError", "NotSPDError", "MultiSystemBatch", "initialize_multi", "Server", "kf_build", "BlockTriDiagData_cpu", "initialize_cpu",
    "ReferenceAlgorithmData", "initialize_reference_algorithm",
    "construct_block_tridiagonal", "SparseCholeskyData", "initialize_sparse_cholesky", "analyze_",
    "autotune", "autotune_lookup", "autotune_save", "autotune_load", "autotune_clear",
]


def _torch():
    import torch
    return torch


def _dtype_code(T):
    torch = _torch()
    if T in (torch.float64, "float64", "Float64", "f64", float):
        return _lib.BSS_F64, torch.float64
    if T in (torch.float32, "float32", "Float32", "f32"):
        return _lib.BSS_F32, torch.float32
    raise ValueError(f"unsupported element type {T!r}: Float32 or Float64")


class _DevView:
    """__cuda_array_interface__ over library memory; keeps the owner alive."""

    def __init__(self, ptr, shape, strides, typestr, owner):
        self._owner = owner
        self.__cuda_array_interface__ = {
            "shape": tuple(int(s) for s in shape),
            "strides": tuple(int(s) for s in strides),
            "typestr": typestr,
            "data": (int(ptr), False),
            "version": 3,
            "stream": None,
        }


class _Handle:
    """Owns a bss_handle*; destroyed when the last tensor view is gone."""

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            if self.ptr:
                _lib.load().bss_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


class _Data:
    def __init__(self, handle: _Handle, torch_dtype, N_user: int):
        torch = _torch()
        L = _lib.load()
        self._h = handle
        N = ctypes.c_int64()
        n = ctypes.c_int64()
        k = ctypes.c_int64()
        dt = ctypes.c_int32()
        _lib.check(L.bss_get_dims(handle.ptr, ctypes.byref(N), ctypes.byref(n), ctypes.byref(k),
                                  ctypes.byref(dt)))
        A = ctypes.c_void_p()
        B = ctypes.c_void_p()
        d = ctypes.c_void_p()
        _lib.check(L.bss_get_tensors(handle.ptr, ctypes.byref(A), ctypes.byref(B), ctypes.byref(d)))
        self.N = N.value
        self.n = n.value
        self.k = k.value
        self.N_user = N_user
        self.dtype = torch_dtype
        es = 8 if torch_dtype == torch.float64 else 4
        ts = "<f8" if es == 8 else "<f4"
        nn = self.n * self.n
        dev = torch.device("cuda", torch.cuda.current_device())
        self.A_tensor = torch.as_tensor(
            _DevView(A.value, (self.n, self.n, self.N), (es, es * self.n, es * nn), ts, handle), device=dev)
        self.B_tensor = torch.as_tensor(
            _DevView(B.value, (self.n, self.n, max(self.N - 1, 0)), (es, es * self.n, es * nn), ts, handle),
            device=dev)
        self.d_tensor = torch.as_tensor(
            _DevView(d.value, (self.n, self.k, self.N), (es, es * self.n, es * self.n * self.k), ts, handle),
            device=dev)
        self.A_list = [self.A_tensor[:, :, i] for i in range(self.N)]
        self.B_list = [self.B_tensor[:, :, i] for i in range(max(self.N - 1, 0))]
        self.d_list = [self.d_tensor[:, :, i] for i in range(self.N)]

    @property
    def handle(self):
        return self._h.ptr


class BlockTriDiagData_batched(_Data):
    """``BlockTriDiagData_batched`` (src/gpu_batched.jl:1-71): N (padded N_use),
    n, A_tensor, B_tensor, d_tensor and the per-block lists.  The per-level
    workspace of the reference struct lives inside the library handle."""


class BlockTriDiagData_seq(_Data):
    """``BlockTriDiagData_seq`` (src/gpu_seq.jl:1-27)."""


def _stream_ptr(stream):
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(int(stream.cuda_stream))


def initialize_batched(N: int, n: int, T=None, M=None, *, k: int = 1, precision: str = "plain",
                       plan: str = "auto", max_refine: int = 10, tol: float = 1e-12,
                       target_partitions: int = 0, seq_cutoff: int = 0, use_graphs: bool = True,
                       coarsest_fp64: bool = False, stream=None) -> BlockTriDiagData_batched:
    """initialize_batched(N, n, T, CuArray) (src/gpu_batched.jl:165-182).

    ``M`` is accepted for signature parity (the reference passes CuArray) and
    ignored.  ``precision="mixed"`` (Float64 only): FP32 factorization with
    FP64 iterative refinement to ``tol``.  ``plan="reference"`` uses the
    reference planner's level sequence; "auto" sizes partitions to the GPU.
    ``use_graphs``: after the first call, factorize!/solve! replay CUDA graphs
    (the mixed solve's refinement loop runs on the device).
    ``coarsest_fp64`` (mixed only): factor and solve the sequential coarsest
    Schur complement in FP64 instead of FP32.
    """
    torch = _torch()
    code, tdt = _dtype_code(torch.float64 if T is None else T)
    o = _lib.default_options()
    o.precision = {"plain": _lib.BSS_PRECISION_PLAIN, "mixed": _lib.BSS_PRECISION_MIXED}[precision]
    o.plan = {"auto": _lib.BSS_PLAN_AUTO, "reference": _lib.BSS_PLAN_REFERENCE}[plan]
    o.max_refine = int(max_refine)
    o.tol = float(tol)
    o.target_partitions = int(target_partitions)
    o.seq_cutoff = int(seq_cutoff)
    o.use_graphs = 1 if use_graphs else 0
    o.coarsest_fp64 = 1 if coarsest_fp64 else 0
    L = _lib.load()
    h = ctypes.c_void_p()
    torch.cuda.current_device()  # make torch bind the device's primary context first
    _lib.check(L.bss_create_batched(int(N), int(n), int(k), code, _stream_ptr(stream), ctypes.byref(o),
                                    ctypes.byref(h)))
    return BlockTriDiagData_batched(_Handle(h.value), tdt, int(N))


def initialize_seq(N: int, n: int, T=None, M=None, *, k: int = 1, stream=None) -> BlockTriDiagData_seq:
    """initialize_seq(N, n, T, CuArray) (src/gpu_seq.jl:45-59)."""
    torch = _torch()
    code, tdt = _dtype_code(torch.float64 if T is None else T)
    L = _lib.load()
    h = ctypes.c_void_p()
    torch.cuda.current_device()
    _lib.check(L.bss_create_seq(int(N), int(n), int(k), code, _stream_ptr(stream), ctypes.byref(h)))
    return BlockTriDiagData_seq(_Handle(h.value), tdt, int(N))


class _RefHandle:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            if self.ptr:
                _lib.load().bss_refalgo_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


class ReferenceAlgorithmData:
    """The reference's batched GPU algorithm restated over cuSOLVER/cuBLAS
    (bss_refalgo_*), for comparison: same tensors as BlockTriDiagData_batched
    (A_tensor, B_tensor, d_tensor column-major views of N_use blocks)."""

    def __init__(self, handle: _RefHandle, torch_dtype):
        torch = _torch()
        L = _lib.load()
        self._h = handle
        N, n, k = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(L.bss_refalgo_get_dims(handle.ptr, ctypes.byref(N), ctypes.byref(n), ctypes.byref(k)))
        A, B, d = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _lib.check(L.bss_refalgo_get_tensors(handle.ptr, ctypes.byref(A), ctypes.byref(B), ctypes.byref(d)))
        self.N, self.n, self.k, self.dtype = N.value, n.value, k.value, torch_dtype
        es = 8 if torch_dtype == torch.float64 else 4
        ts = "<f8" if es == 8 else "<f4"
        nn = self.n * self.n
        dev = torch.device("cuda", torch.cuda.current_device())
        self.A_tensor = torch.as_tensor(
            _DevView(A.value, (self.n, self.n, self.N), (es, es * self.n, es * nn), ts, handle), device=dev)
        self.B_tensor = torch.as_tensor(
            _DevView(B.value, (self.n, self.n, max(self.N - 1, 0)), (es, es * self.n, es * nn), ts, handle),
            device=dev)
        self.d_tensor = torch.as_tensor(
            _DevView(d.value, (self.n, self.k, self.N), (es, es * self.n, es * self.n * self.k), ts, handle),
            device=dev)

    @property
    def handle(self):
        return self._h.ptr


def initialize_reference_algorithm(N: int, n: int, T=None, *, k: int = 1, stream=None) -> ReferenceAlgorithmData:
    """The reference's own algorithm (src/gpu_batched.jl over batched
    cuSOLVER/cuBLAS) on this GPU, for timing comparisons."""
    torch = _torch()
    code, tdt = _dtype_code(torch.float64 if T is None else T)
    h = ctypes.c_void_p()
    torch.cuda.current_device()
    _lib.check(_lib.load().bss_refalgo_create(int(N), int(n), int(k), code, _stream_ptr(stream), ctypes.byref(h)))
    return ReferenceAlgorithmData(_RefHandle(h.value), tdt)


def _blocks_colmajor(X, n, count):
    """Device tensor (n, n, count) whose blocks are column-major in memory:
    element (r, c, i) at i n^2 + c n + r (a copy only if X is laid out
    otherwise)."""
    if tuple(X.shape) != (n, n, count):
        raise ValueError(f"expected blocks of shape ({n}, {n}, {count}), got {tuple(X.shape)}")
    if count > 0 and tuple(X.stride()) != (1, n, n * n):
        X = X.permute(2, 1, 0).contiguous().permute(2, 1, 0)
    return X


def construct_block_tridiagonal(A_tensor, B_tensor, d_tensor=None, *, stream=None):
    """construct_block_tridiagonal(A_list, B_list, d_list)
    (benchmark/utils.jl:59-103) on the device.

    A_tensor (n x n x N) and B_tensor (n x n x (N-1)) are CUDA tensors of the
    blocks (A_tensor[:, :, i] = A_i).  Returns ``(M, d_vec)``: M the
    (N n) x (N n) matrix with A_i on the diagonal, B_i at block (i, i+1) and
    B_i^T at block (i+1, i) as a torch sparse CSR tensor with int32 indices,
    every entry of every block stored and the values copied bit for bit
    (bss_csr_assemble); d_vec = vcat(d_list...), the (N n) x k right-hand
    side, or None without d_tensor."""
    torch = _torch()
    n, N = int(A_tensor.shape[0]), int(A_tensor.shape[2])
    code, tdt = _dtype_code(A_tensor.dtype)
    if not A_tensor.is_cuda:
        raise ValueError("construct_block_tridiagonal: A_tensor must be a CUDA tensor")
    A = _blocks_colmajor(A_tensor, n, N)
    B = _blocks_colmajor(B_tensor.to(dtype=tdt), n, N - 1)
    L = _lib.load()
    nnz = int(L.bss_csr_nnz(N, n))
    dev = A.device
    crow = torch.empty(N * n + 1, dtype=torch.int32, device=dev)
    col = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    val = torch.empty(max(nnz, 1), dtype=tdt, device=dev)
    bptr = B.data_ptr() if N > 1 else 0
    _lib.check(L.bss_csr_assemble(N, n, code, ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(bptr),
                                  ctypes.c_void_p(crow.data_ptr()), ctypes.c_void_p(col.data_ptr()),
                                  ctypes.c_void_p(val.data_ptr()), _stream_ptr(stream)))
    M = torch.sparse_csr_tensor(crow, col[:nnz], val[:nnz], size=(N * n, N * n))
    d_vec = None
    if d_tensor is not None:
        k = int(d_tensor.shape[1])
        d_vec = d_tensor.permute(2, 0, 1).reshape(N * n, k)
    return M, d_vec


class _SpHandle:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            if self.ptr:
                _lib.load().bss_spchol_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


class SparseCholeskyData:
    """The reference's sparse direct-solver comparison
    (benchmark/benchmark_gpu.jl:75-117) on this GPU: the assembled CSR
    matrix of construct_block_tridiagonal factored by a general sparse
    Cholesky (bss_spchol_*; cuSOLVER's GPU csrchol stands in for cuDSS,
    which this toolkit lacks).  A_tensor, B_tensor, d_tensor as for
    BlockTriDiagData_batched (no padding); ``csr()`` is a zero-copy sparse
    CSR view of the assembled matrix after ``analyze_`` or ``factorize_``."""

    def __init__(self, handle: _SpHandle, torch_dtype):
        torch = _torch()
        L = _lib.load()
        self._h = handle
        N, n, k = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(L.bss_spchol_get_dims(handle.ptr, ctypes.byref(N), ctypes.byref(n), ctypes.byref(k)))
        A, B, d = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _lib.check(L.bss_spchol_get_tensors(handle.ptr, ctypes.byref(A), ctypes.byref(B), ctypes.byref(d)))
        self.N, self.n, self.k, self.dtype = N.value, n.value, k.value, torch_dtype
        es = 8 if torch_dtype == torch.float64 else 4
        self._ts = "<f8" if es == 8 else "<f4"
        self._es = es
        nn = self.n * self.n
        dev = torch.device("cuda", torch.cuda.current_device())
        self._dev = dev
        self.A_tensor = torch.as_tensor(
            _DevView(A.value, (self.n, self.n, self.N), (es, es * self.n, es * nn), self._ts, handle), device=dev)
        self.B_tensor = torch.as_tensor(
            _DevView(B.value, (self.n, self.n, max(self.N - 1, 0)), (es, es * self.n, es * nn), self._ts, handle),
            device=dev)
        self.d_tensor = torch.as_tensor(
            _DevView(d.value, (self.n, self.k, self.N), (es, es * self.n, es * self.n * self.k), self._ts, handle),
            device=dev)

    @property
    def handle(self):
        return self._h.ptr

    def csr(self):
        torch = _torch()
        rp, ci, v, nnz = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_int64()
        _lib.check(_lib.load().bss_spchol_get_csr(self.handle, ctypes.byref(rp), ctypes.byref(ci), ctypes.byref(v),
                                                  ctypes.byref(nnz)))
        rows = self.N * self.n
        crow = torch.as_tensor(_DevView(rp.value, (rows + 1,), (4,), "<i4", self._h), device=self._dev)
        col = torch.as_tensor(_DevView(ci.value, (nnz.value,), (4,), "<i4", self._h), device=self._dev)
        val = torch.as_tensor(_DevView(v.value, (nnz.value,), (self._es,), self._ts, self._h), device=self._dev)
        return torch.sparse_csr_tensor(crow, col, val, size=(rows, rows))


def initialize_sparse_cholesky(N: int, n: int, T=None, *, k: int = 1, stream=None) -> SparseCholeskyData:
    """Sparse direct-solver comparison (benchmark/benchmark_gpu.jl:75-117):
    same tensors as initialize_batched; analyze_/factorize_/solve_ run the
    analysis, factorization and solve phases on the assembled CSR matrix."""
    torch = _torch()
    code, tdt = _dtype_code(torch.float64 if T is None else T)
    h = ctypes.c_void_p()
    torch.cuda.current_device()
    _lib.check(_lib.load().bss_spchol_create(int(N), int(n), int(k), code, _stream_ptr(stream), ctypes.byref(h)))
    return SparseCholeskyData(_SpHandle(h.value), tdt)


def analyze_(data: SparseCholeskyData) -> None:
    """The analysis phase of the sparse comparison (cudss("analysis", ...),
    benchmark/benchmark_gpu.jl:93): assemble the CSR matrix from A_tensor /
    B_tensor and run the symbolic factorization."""
    _lib.check(_lib.load().bss_spchol_analyze(data.handle))


class _CpuHandle:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            if self.ptr:
                _lib.load().bss_cpu_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


class BlockTriDiagData_cpu:
    """``BlockTriDiagData_cpu`` (src/cpu.jl:1-10): N, n and A_list, B_list,
    d_list -- numpy views of the handle's host memory (column-major blocks,
    also exposed whole as A_tensor (n,n,N), B_tensor, d_tensor)."""

    def __init__(self, handle: _CpuHandle, N, n, k, np_dtype):
        import numpy as np
        self._h = handle
        self.N, self.n, self.k = N, n, k
        A = ctypes.c_void_p()
        B = ctypes.c_void_p()
        d = ctypes.c_void_p()
        _lib.check(_lib.load().bss_cpu_get_tensors(handle.ptr, ctypes.byref(A), ctypes.byref(B), ctypes.byref(d)))
        es = np.dtype(np_dtype).itemsize
        ct = ctypes.c_double if es == 8 else ctypes.c_float

        def view(ptr, r, c, cnt):
            buf = (ct * (r * c * max(cnt, 1))).from_address(ptr)
            return np.ndarray((r, c, cnt), dtype=np_dtype, buffer=buf, strides=(es, es * r, es * r * c))

        self.A_tensor = view(A.value, n, n, N)
        self.B_tensor = view(B.value, n, n, N - 1)
        self.d_tensor = view(d.value, n, k, N)
        self.A_list = [self.A_tensor[:, :, i] for i in range(N)]
        self.B_list = [self.B_tensor[:, :, i] for i in range(N - 1)]
        self.d_list = [self.d_tensor[:, :, i] for i in range(N)]

    @property
    def handle(self):
        return self._h.ptr


def initialize_cpu(N: int, n: int, T=None, *, k: int = 1) -> BlockTriDiagData_cpu:
    """initialize_cpu(N, n, T) (src/cpu.jl:12-29): zeroed host blocks."""
    import numpy as np
    if T in (None, float, "float64", "Float64", "f64", np.float64):
        code, npt = _lib.BSS_F64, np.float64
    elif T in ("float32", "Float32", "f32", np.float32):
        code, npt = _lib.BSS_F32, np.float32
    else:
        torch = _torch()
        code = _dtype_code(T)[0]
        npt = np.float64 if code == _lib.BSS_F64 else np.float32
    h = ctypes.c_void_p()
    _lib.check(_lib.load().bss_cpu_create(int(N), int(n), int(k), code, ctypes.byref(h)))
    return BlockTriDiagData_cpu(_CpuHandle(h.value), int(N), int(n), int(k), npt)


def factorize_(data, check: bool = False) -> None:
    """factorize!(data) (src/gpu_batched.jl:184-227 / src/gpu_seq.jl:61-71 /
    src/cpu.jl:31-40).  GPU handles: asynchronous on the handle's stream;
    ``check=True`` waits and raises NotSPDError if a pivot failed.  CPU
    data: synchronous, raises NotSPDError on a failed pivot."""
    if isinstance(data, BlockTriDiagData_cpu):
        _lib.check(_lib.load().bss_cpu_factorize(data.handle))
        return
    if isinstance(data, ReferenceAlgorithmData):
        _lib.check(_lib.load().bss_refalgo_factorize(data.handle))
        return
    if isinstance(data, SparseCholeskyData):
        _lib.check(_lib.load().bss_spchol_factorize(data.handle))
        return
    _lib.check(_lib.load().bss_factorize(data.handle))
    if check:
        synchronize(data)


def solve_(data, check: bool = False) -> None:
    """solve!(data) (src/gpu_batched.jl:229-258 / src/gpu_seq.jl:73-84 /
    src/cpu.jl:42-50): d_tensor <- A^{-1} d_tensor."""
    if isinstance(data, BlockTriDiagData_cpu):
        _lib.check(_lib.load().bss_cpu_solve(data.handle))
        return
    if isinstance(data, ReferenceAlgorithmData):
        _lib.check(_lib.load().bss_refalgo_solve(data.handle))
        return
    if isinstance(data, SparseCholeskyData):
        _lib.check(_lib.load().bss_spchol_solve(data.handle))
        return
    _lib.check(_lib.load().bss_solve(data.handle))
    if check:
        synchronize(data)


factorize = factorize_
solve = solve_


def _host_blocks(X, dims, torch_dtype, what, writable=False):
    """Address of a dense host array of `count` column-major a x b blocks
    (dims = (a, b, count)): shape (a, b, count) with column-major strides
    (Julia's layout) or the same memory as a row-major (count, b, a) array.
    numpy arrays or CPU torch tensors; nothing is copied."""
    torch = _torch()
    import numpy as np
    a, b, cnt = (int(v) for v in dims)
    want_f, want_c = (a, b, cnt), (cnt, b, a)
    if isinstance(X, torch.Tensor):
        if X.device.type != "cpu":
            raise ValueError(f"{what}: a host array is required, got a tensor on {X.device}")
        if X.dtype != torch_dtype:
            raise ValueError(f"{what}: dtype {X.dtype}, the handle holds {torch_dtype}")
        shape, st = tuple(X.shape), tuple(X.stride())
        ok = (shape == want_c and X.is_contiguous()) or (shape == want_f and st == (1, a, a * b))
        ptr = X.data_ptr()
    else:
        if not isinstance(X, np.ndarray):
            raise ValueError(f"{what}: expected a numpy array or a CPU torch tensor")
        npdt = np.float64 if torch_dtype == torch.float64 else np.float32
        if X.dtype != npdt:
            raise ValueError(f"{what}: dtype {X.dtype}, the handle holds {np.dtype(npdt)}")
        if writable and not X.flags.writeable:
            raise ValueError(f"{what}: array is read-only")
        ok = (X.shape == want_c and X.flags.c_contiguous) or (X.shape == want_f and X.flags.f_contiguous)
        ptr = X.ctypes.data
    if not ok:
        raise ValueError(f"{what}: expected a dense host array of shape {want_f} (column-major) or {want_c} "
                         f"(row-major), got {tuple(X.shape)}")
    return ptr


def upload(data: _Data, A=None, B=None, d=None, *, upper: bool = False) -> int:
    """Host arrays -> the handle's A/B/d tensors (bss_upload), the
    ``copyto!(data.A_tensor, A)`` ... of the reference's callers
    (benchmark/benchmark_gpu.jl:129-131) for host data.  A: N blocks n x n,
    B: N-1 blocks, d: N blocks n x k (N the size the handle was created
    with), column-major (n, n, N) or row-major (N, n, n) host arrays of the
    handle's dtype; page-locked memory (``tensor.pin_memory()``) makes the
    copies asynchronous on the handle's stream, and then the arrays must
    stay alive and unchanged until the stream reaches them.

    ``upper=True``: only the upper triangle of each A_i defines the block
    (the triangle the reference's potrf(FILL_MODE_UPPER) reads); it is
    mirrored into the lower one on the device.  Returns the bytes read from
    host memory."""
    n, k, N = data.n, data.k, data.N_user
    pa = _host_blocks(A, (n, n, N), data.dtype, "A") if A is not None else None
    pb = _host_blocks(B, (n, n, N - 1), data.dtype, "B") if B is not None and N > 1 else None
    pd = _host_blocks(d, (n, k, N), data.dtype, "d") if d is not None else None
    moved = ctypes.c_int64()
    flag = _lib.BSS_UPLOAD_UPPER if upper else _lib.BSS_UPLOAD_FULL
    _lib.check(_lib.load().bss_upload(data.handle, pa, pb, pd, flag, ctypes.byref(moved)))
    return moved.value


def download(data: _Data, x) -> None:
    """d_tensor's first N blocks (the solution after solve!) -> host array x
    (n x k x N, layouts as in upload); asynchronous on the handle's stream
    when x is page-locked: complete after synchronize(data)."""
    ptr = _host_blocks(x, (data.n, data.k, data.N_user), data.dtype, "x", writable=True)
    _lib.check(_lib.load().bss_download(data.handle, ptr))


def synchronize(data: _Data) -> None:
    """Wait for the handle's stream; raise on a failed pivot or on a
    refinement that missed its tolerance."""
    _lib.check(_lib.load().bss_synchronize(data.handle))


def get_info(data: _Data) -> dict:
    inf = _lib.Info()
    _lib.check(_lib.load().bss_get_info(data.handle, ctypes.byref(inf)))
    return {k: getattr(inf, k) for k, _ in _lib.Info._fields_}


def residual(A_tensor, B_tensor, x_tensor, d_tensor, stream=None) -> float:
    """||d - T x||_inf / (||T||_inf ||x||_inf + ||d||_inf) on the device (FP64
    accumulation) for column-major (n,n,N)/(n,n,N-1)/(n,k,N) tensors."""
    torch = _torch()
    n, _, N = A_tensor.shape
    k = x_tensor.shape[1]
    code, _ = _dtype_code(A_tensor.dtype)

    def colmajor(t):
        return t.stride(0) == 1 and t.stride(1) == t.shape[0] and t.stride(2) == t.shape[0] * t.shape[1]

    for t in (A_tensor, x_tensor, d_tensor):
        if not colmajor(t) or not t.is_cuda:
            raise ValueError("tensors must be column-major CUDA tensors")
    out = ctypes.c_double()
    Bp = B_tensor.data_ptr() if B_tensor.numel() else A_tensor.data_ptr()
    _lib.check(_lib.load().bss_residual(N, n, k, code, ctypes.c_void_p(A_tensor.data_ptr()), ctypes.c_void_p(Bp),
                                        ctypes.c_void_p(x_tensor.data_ptr()), ctypes.c_void_p(d_tensor.data_ptr()),
                                        _stream_ptr(stream), ctypes.byref(out)))
    return out.value


class _BatchHandle:
    """Owns a bss_batch*; destroyed when the last tensor view is gone."""

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            if self.ptr:
                _lib.load().bss_batch_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


class MultiSystemBatch:
    """Many independent block-tridiagonal systems of their own N, n and k,
    factorized and solved together (no counterpart in the reference).

    ``systems[s]`` has ``A_tensor`` (n x n x N), ``B_tensor`` (n x n x (N-1))
    and ``d_tensor`` (n x k x N): column-major views of library memory, laid
    out like a single system's.  ``factorize()`` / ``solve()`` run every
    system; ``d_tensor`` then holds each system's solution."""

    class _System:
        pass

    def __init__(self, handle: _BatchHandle, nsys: int, torch_dtype):
        torch = _torch()
        L = _lib.load()
        self._h = handle
        self.dtype = torch_dtype
        es = 8 if torch_dtype == torch.float64 else 4
        ts = "<f8" if es == 8 else "<f4"
        dev = torch.device("cuda", torch.cuda.current_device())
        self.systems = []
        for s in range(nsys):
            N = ctypes.c_int64()
            n = ctypes.c_int64()
            k = ctypes.c_int64()
            _lib.check(L.bss_batch_get_dims(handle.ptr, s, ctypes.byref(N), ctypes.byref(n), ctypes.byref(k)))
            A = ctypes.c_void_p()
            B = ctypes.c_void_p()
            d = ctypes.c_void_p()
            _lib.check(L.bss_batch_get_tensors(handle.ptr, s, ctypes.byref(A), ctypes.byref(B), ctypes.byref(d)))
            N, n, k = N.value, n.value, k.value
            nn = n * n
            sysv = MultiSystemBatch._System()
            sysv.N, sysv.n, sysv.k, sysv.dtype = N, n, k, torch_dtype
            sysv.A_tensor = torch.as_tensor(
                _DevView(A.value, (n, n, N), (es, es * n, es * nn), ts, handle), device=dev)
            sysv.B_tensor = torch.as_tensor(
                _DevView(B.value, (n, n, max(N - 1, 0)), (es, es * n, es * nn), ts, handle), device=dev)
            sysv.d_tensor = torch.as_tensor(
                _DevView(d.value, (n, k, N), (es, es * n, es * n * k), ts, handle), device=dev)
            self.systems.append(sysv)

    @property
    def handle(self):
        return self._h.ptr

    def __len__(self):
        return len(self.systems)

    def factorize(self, check: bool = False) -> None:
        _lib.check(_lib.load().bss_batch_factorize(self.handle))
        if check:
            self.synchronize()

    def solve(self, check: bool = False) -> None:
        _lib.check(_lib.load().bss_batch_solve(self.handle))
        if check:
            self.synchronize()

    def synchronize(self) -> None:
        _lib.check(_lib.load().bss_batch_synchronize(self.handle))

    def info(self, s: int) -> dict:
        inf = _lib.Info()
        _lib.check(_lib.load().bss_batch_get_info(self.handle, int(s), ctypes.byref(inf)))
        return {k: getattr(inf, k) for k, _ in _lib.Info._fields_}


def initialize_multi(Ns, ns, ks=None, T=None, *, precision: str = "plain", max_refine: int = 10,
                     tol: float = 1e-12, use_graphs: bool = True, stream=None) -> MultiSystemBatch:
    """Create a batch of independent systems: system s has Ns[s] blocks of
    size ns[s] (<= 64) and ks[s] right-hand sides (default 1)."""
    torch = _torch()
    code, tdt = _dtype_code(torch.float64 if T is None else T)
    nsys = len(Ns)
    if ks is None:
        ks = [1] * nsys
    if not (len(ns) == nsys and len(ks) == nsys) or nsys < 1:
        raise ValueError("Ns, ns and ks must be non-empty and of equal length")
    o = _lib.default_options()
    o.precision = {"plain": _lib.BSS_PRECISION_PLAIN, "mixed": _lib.BSS_PRECISION_MIXED}[precision]
    o.max_refine = int(max_refine)
    o.tol = float(tol)
    o.use_graphs = 1 if use_graphs else 0
    arr = ctypes.c_int64 * nsys
    L = _lib.load()
    h = ctypes.c_void_p()
    torch.cuda.current_device()
    _lib.check(L.bss_batch_create(nsys, arr(*map(int, Ns)), arr(*map(int, ns)), arr(*map(int, ks)), code,
                                  _stream_ptr(stream), ctypes.byref(o), ctypes.byref(h)))
    return MultiSystemBatch(_BatchHandle(h.value), nsys, tdt)


def plan_reference(N: int):
    return _lib.plan_reference(N)


def _tune_key(n, T, precision):
    code, _ = _dtype_code(_torch().float64 if T is None else T)
    prec = {"plain": _lib.BSS_PRECISION_PLAIN, "mixed": _lib.BSS_PRECISION_MIXED}[precision]
    return int(n), code, prec


def autotune(n, T=None, precision="mixed", N_probe=16384) -> dict:
    """Time candidate plans for block size n and keep the fastest (see
    bss_autotune in include/bss.h); later handles, batches and server
    requests with default options use it."""
    e = _lib.TuneEntry()
    n, code, prec = _tune_key(n, T, precision)
    _lib.check(_lib.load().bss_autotune(n, code, prec, int(N_probe), ctypes.byref(e)))
    return {k: getattr(e, k) for k, _ in _lib.TuneEntry._fields_}


def autotune_lookup(n, T=None, precision="mixed"):
    e = _lib.TuneEntry()
    n, code, prec = _tune_key(n, T, precision)
    rc = _lib.load().bss_autotune_lookup(n, code, prec, ctypes.byref(e))
    return None if rc else {k: getattr(e, k) for k, _ in _lib.TuneEntry._fields_}


def autotune_save(path):
    _lib.check(_lib.load().bss_autotune_save(str(path).encode()))


def autotune_load(path):
    _lib.check(_lib.load().bss_autotune_load(str(path).encode()))


def autotune_clear():
    _lib.load().bss_autotune_clear()


def _ptr(a):
    """Address of a host buffer: a C-contiguous float64 numpy array or a CPU
    torch tensor (page-locked ones make the server's copies asynchronous)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        if a.dtype != _torch().float64 or not a.is_contiguous():
            raise ValueError("host tensors must be contiguous float64")
        return ctypes.c_void_p(a.data_ptr())
    import numpy as np
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("host arrays must be C-contiguous float64")
    return ctypes.c_void_p(a.ctypes.data)


def kf_build(F, H, Qinv, Rinv, y, A_out, B_out, d_out, P0inv=None, x0=None, stream=None) -> None:
    """Kalman-smoother normal equations on the device (build_kf_blocks,
    benchmark/benchmark_kf.jl:105-154): column-major CUDA float64 tensors
    F (n,n), H (m,n), Qinv (n,n), Rinv (m,m), y (m,k,N) -> A (n,n,N),
    B (n,n,N-1), d (n,k,N)."""
    m, k, N = y.shape
    n = F.shape[0]
    dp = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    _lib.check(_lib.load().bss_kf_build(N, n, m, k, dp(F), dp(H), dp(Qinv), dp(Rinv), dp(P0inv), dp(x0), dp(y),
                                        dp(A_out), dp(B_out) if N > 1 else None, dp(d_out), _stream_ptr(stream)))


class Server:
    """Request server over the C ABI (bss_server_*): continuous batching of
    independent solves under an HBM budget, resident factors for repeat
    right-hand sides, p50/p99 latency.  Host buffers (inputs and outputs)
    must stay alive and unchanged until ``wait`` returns for the request;
    this class keeps references to them until then."""

    def __init__(self, hbm_budget_bytes=None, streams=None, max_inflight=None, precision="mixed",
                 max_refine=None, tol=None):
        L = _lib.load()
        o = _lib.ServerOptions()
        L.bss_server_default_options(ctypes.byref(o))
        if hbm_budget_bytes is not None:
            o.hbm_budget_bytes = int(hbm_budget_bytes)
        if streams is not None:
            o.streams = int(streams)
        if max_inflight is not None:
            o.max_inflight = int(max_inflight)
        o.precision = {"plain": _lib.BSS_PRECISION_PLAIN, "mixed": _lib.BSS_PRECISION_MIXED}[precision]
        if max_refine is not None:
            o.max_refine = int(max_refine)
        if tol is not None:
            o.tol = float(tol)
        _torch().cuda.current_device()
        h = ctypes.c_void_p()
        _lib.check(L.bss_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h.value
        self._keep = {}

    def close(self):
        if self._h:
            _lib.load().bss_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, A, B, d, x_out, keep=False):
        """A (N,n,n) storage order (block i column-major = numpy (N, c, r)),
        B (N-1,n,n), d (N,k,n) -> x_out (N,k,n).  Returns (request, factor)."""
        N, n = A.shape[0], A.shape[1]
        k = d.shape[1]
        rid, fid = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(_lib.load().bss_server_submit(self._h, N, n, k, _ptr(A), _ptr(B) if N > 1 else None, _ptr(d),
                                                 1 if keep else 0, _ptr(x_out), ctypes.byref(rid),
                                                 ctypes.byref(fid)))
        self._keep[rid.value] = (A, B, d, x_out)
        return rid.value, fid.value

    def submit_kalman(self, F, H, Qinv, Rinv, y, x_out, P0inv=None, x0=None, keep=False):
        """Column-major host arrays: F (n,n) as numpy (c, r), H (m,n) as (n, m),
        Qinv, Rinv, y (m,k,N) as numpy (N, k, m) -> x_out (N, k, n)."""
        N, k, m = y.shape
        n = F.shape[0]
        rid, fid = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(_lib.load().bss_server_submit_kalman(self._h, N, n, m, k, _ptr(F), _ptr(H), _ptr(Qinv),
                                                        _ptr(Rinv), _ptr(P0inv), _ptr(x0), _ptr(y),
                                                        1 if keep else 0, _ptr(x_out), ctypes.byref(rid),
                                                        ctypes.byref(fid)))
        self._keep[rid.value] = (F, H, Qinv, Rinv, P0inv, x0, y, x_out)
        return rid.value, fid.value

    def submit_rhs(self, factor_id, d_or_y, x_out):
        rid = ctypes.c_uint64()
        _lib.check(_lib.load().bss_server_submit_rhs(self._h, int(factor_id), _ptr(d_or_y), _ptr(x_out),
                                                     ctypes.byref(rid)))
        self._keep[rid.value] = (d_or_y, x_out)
        return rid.value

    def wait(self, request_id, check=True) -> dict:
        inf = _lib.RequestInfo()
        rc = _lib.load().bss_server_wait(self._h, int(request_id), ctypes.byref(inf))
        self._keep.pop(int(request_id), None)
        out = {k: getattr(inf, k) for k, _ in _lib.RequestInfo._fields_}
        if check:
            _lib.check(rc)
        return out

    def poll(self, request_id) -> bool:
        done = ctypes.c_int32()
        _lib.check(_lib.load().bss_server_poll(self._h, int(request_id), ctypes.byref(done)))
        return bool(done.value)

    def release(self, factor_id) -> None:
        _lib.check(_lib.load().bss_server_release(self._h, int(factor_id)))

    def stats(self) -> dict:
        st = _lib.ServerStats()
        _lib.check(_lib.load().bss_server_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def reset_stats(self) -> None:
        _lib.check(_lib.load().bss_server_reset_stats(self._h))


def colmajor_empty(shape, dtype, device="cuda"):
    """A torch tensor with Julia column-major strides (shape (r, c, N))."""
    torch = _torch()
    r, c, N = shape
    return torch.empty((N, c, r), dtype=dtype, device=device).permute(2, 1, 0)
