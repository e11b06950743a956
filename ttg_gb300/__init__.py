"""ttg_gb300 — GB300-native (sm_103a) device-task path of TTG's tiled Cholesky.

The compute lives in `libgbx_potrf.so` (C ABI, include/gbx_potrf.h). This module is a thin
ctypes front end for Python callers (tests, benchmark): it loads the in-tree library, declares
the signatures and turns status codes into exceptions. Device memory and streams come from
PyTorch; only raw pointers cross the boundary.

There is no fallback: if the library is missing or fails to load, every call raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbx_potrf.so")

GBX_OK = 0
GBX_ERR_ARG = -1
GBX_ERR_CUDA = -2
GBX_ERR_TIMEOUT = -3
GBX_ERR_WORKSPACE = -4
GBX_ERR_NOCONV = -5
GBX_ERR_NOALLOC_LIMIT = -6
PREC = {"bf16": 0, "fp16": 1, "fp8": 2}

_ERRNAMES = {GBX_ERR_ARG: "invalid argument", GBX_ERR_CUDA: "CUDA runtime error",
             GBX_ERR_TIMEOUT: "device-side wait timed out", GBX_ERR_WORKSPACE: "workspace too small",
             GBX_ERR_NOCONV: "refinement did not reach the tolerance",
             GBX_ERR_NOALLOC_LIMIT: "problem exceeds the allocation-free entry point's scratch"}

_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_sz = ctypes.c_size_t
_szp = ctypes.POINTER(ctypes.c_size_t)
_d = ctypes.c_double
_u64 = ctypes.c_uint64
_ull = ctypes.c_ulonglong

# name -> (restype, argtypes)
SIGNATURES = {
    "gbx_version": (_i, []),
    "gbx_built_arch": (_i, []),
    "gbx_set_wait_timeout_ns": (None, [_u64]),
    "gbx_set_trace_buffer": (None, [_vp, _i]),
    "gbx_get_wait_timeout_ns": (_u64, []),
    "gbx_dpotrf_tile_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_dpotrf_tile": (_i, [_i, _vp, _i, _vp, _sz, _vp, _vp]),
    "gbx_dtrsm_rlt_tile": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dsyrk_ln_tile": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dgemm_nt_tile": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dtrsm_rln_tile": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dgemm_nn_tile": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_taskq_create": (_i, [ctypes.POINTER(_vp)]),
    "gbx_taskq_destroy": (_i, [_vp]),
    "gbx_taskq_stream": (_vp, [_vp]),
    "gbx_taskq_pending": (ctypes.c_longlong, [_vp]),
    "gbx_taskq_run": (_i, [_vp, _vp]),
    "gbx_taskq_status": (_i, [_vp, _vp]),
    "gbx_dpotrf_tiled_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_set_dag_block_edge": (_i, [_i]),
    "gbx_set_fp64_update": (_i, [_i]),
    "gbx_get_fp64_update": (_i, []),
    "gbx_dpotrf_tiled": (_i, [_i, _i, _vp, _vp, _sz, _vp]),
    "gbx_dpotrf_tiled_status": (_i, [_vp, _vp]),
    "gbx_dpotrs_tiled": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dplgsy_tiled": (_i, [_i, _i, _d, _ull, _vp, _vp]),
    "gbx_dgen_uniform_sym_tiled": (_i, [_i, _i, _ull, _d, _vp, _vp]),
    "gbx_dplgsy_tile": (_i, [_d, _i, _i, _vp, _i, _i, _i, _i, _ull, _vp]),
    "gbx_dag_timeout_selftest": (_i, [_i, _vp, _vp, _sz, _u64, _vp]),
    "gbx_dpotrf_tiled_noalloc": (_i, [_i, _i, _vp, _vp, _vp]),
    "gbx_gemm_bf16_nt_f32": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _vp]),
    "gbx_dgen_lowrank_sym_tiled": (_i, [_i, _i, _vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "gbx_potrf_mixed_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_potrf_mixed": (_i, [_i, _i, _vp, _vp, _i, _d, _d, _vp, _sz, _vp]),
    "gbx_potrf_mixed_info": (_i, [_vp, _i, _i, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int), _vp]),
    "gbx_spotri_diag": (_i, [_i, _i, _vp, _vp, _vp]),
    "gbx_sprecond": (_i, [_i, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "gbx_dsymm_tiled": (_i, [_i, _i, _vp, _i, _d, _vp, _d, _vp, _vp]),
    "gbx_dposv_mixed_bufferSize": (_i, [_i, _i, _i, _szp]),
    "gbx_batched_order": (_i, [_i, _vp, _vp]),
    "gbx_dgen_uniform_sym_batched": (_i, [_i, _vp, _vp, _ull, _vp, _vp]),
    "gbx_dposv_batched": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _sz, _vp]),
    "gbx_dposv_batched_ex": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp, _i, _vp, _sz, _vp]),
    "gbx_dposv_mixed": (_i, [_i, _i, _vp, _i, _vp, _vp, _i, _d, _d, _i, _vp, _vp, _sz, _vp, _vp]),
    "gbx_dpotri_tiled_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_dpotri_tiled": (_i, [_i, _i, _vp, _vp, _sz, _vp]),
    "gbx_split_f64": (_i, [_vp, _vp, _vp, ctypes.c_longlong, _vp]),
    "gbx_dag_task": (ctypes.c_longlong, [_i, ctypes.c_longlong, _vp]),
    "gbx_dag_task_lead": (ctypes.c_longlong, [_i, ctypes.c_longlong, ctypes.c_longlong, _vp]),
    "gbx_set_dag_lead": (_i, [ctypes.c_longlong]),
    "gbx_mixed_task": (ctypes.c_longlong, [_i, ctypes.c_longlong, _vp]),
    "gbx_dposv_tiled_host_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_dposv_tiled_host": (_i, [_i, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "gbx_potrf_mixed_batched_bufferSize": (_i, [_i, _vp, _i, _szp]),
    "gbx_potrf_mixed_batched": (_i, [_i, _vp, _i, _vp, _vp, _i, _d, _d, _vp, _vp, _sz, _vp]),
    "gbx_potrf_mixed_batched_info": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp, _vp]),
    "gbx_dposv_mixed_batched_bufferSize": (_i, [_i, _vp, _i, _i, _szp]),
    "gbx_dposv_mixed_batched": (_i, [_i, _vp, _i, _vp, _i, _vp, _vp, _i, _d, _d, _i, _vp, _vp, _sz, _vp, _vp]),
    "gbx_dposv_mixed_batched_plan": (_i, [_i, _vp, _i, _i, _i, _i, _vp, _sz, _vp]),
    "gbx_dposv_mixed_batched_exec": (_i, [_i, _vp, _i, _vp, _i, _vp, _vp, _i, _d, _d, _i, _vp, _vp, _sz, _vp]),
    "gbx_dposv_mixed_batched_result": (_i, [_i, _vp, _i, _i, _d, _vp, _vp, _vp]),
}


class GbxError(RuntimeError):
    def __init__(self, fn, code):
        self.code = code
        super().__init__("%s failed: %s (%d)" % (fn, _ERRNAMES.get(code, "status"), code))


class NotPositiveDefinite(RuntimeError):
    """A POTRF pivot was not positive; `info` is its 1-based global index (LAPACK convention)."""

    def __init__(self, info):
        self.info = info
        super().__init__("matrix is not positive definite: pivot %d" % info)


def lib():
    """The loaded C-ABI library. Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgbx_potrf.so is not built: run __graft_entry__.build() "
                               "(or python ttg_gb300/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def call(name, *args):
    """Calls a C-ABI function and raises GbxError on a negative status. Returns the status."""
    st = getattr(lib(), name)(*args)
    if isinstance(st, int) and st < 0:
        raise GbxError(name, st)
    return st


# ---- helpers over torch tensors -------------------------------------------------------------
def _stream(stream):
    import torch
    if stream is None:
        return _vp(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return _vp(stream)
    return _vp(stream.cuda_stream)


def _ptr(t):
    return _vp(t.data_ptr())


def ntiles(N, NB):
    return (N + NB - 1) // NB


def tiled_numel(N, NB):
    nt = ntiles(N, NB)
    return nt * (nt + 1) // 2 * NB * NB


def potrf_workspace_bytes(N, NB):
    b = _sz(0)
    call("gbx_dpotrf_tiled_bufferSize", N, NB, ctypes.byref(b))
    return b.value


def potrf_tiled(tiles, N, NB, workspace=None, stream=None, check=True):
    """Factorises a tile-major lower FP64 matrix (CUDA tensor) in place on the device.

    With check=True the stream is synchronised and a failing pivot raises NotPositiveDefinite.
    Returns the workspace tensor (reuse it across calls)."""
    import torch
    need = potrf_workspace_bytes(N, NB)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=tiles.device)
    s = _stream(stream)
    call("gbx_dpotrf_tiled", N, NB, _ptr(tiles), _ptr(workspace), need, s)
    if check:
        st = call("gbx_dpotrf_tiled_status", _ptr(workspace), s)
        if st > 0:
            raise NotPositiveDefinite(st)
    return workspace


def potrf_status(workspace, stream=None):
    return call("gbx_dpotrf_tiled_status", _ptr(workspace), _stream(stream))


def potrs_tiled(tiles, N, NB, B, stream=None):
    """Solves (L L^T) X = B in place; B is an (nrhs, N) row-major CUDA tensor (= column-major N x nrhs)."""
    nrhs = 1 if B.dim() == 1 else B.shape[0]
    call("gbx_dpotrs_tiled", N, NB, _ptr(tiles), nrhs, _ptr(B), N, _stream(stream))
    return B


def gen_uniform_sym(tiles, N, NB, seed=42, shift=None, stream=None):
    call("gbx_dgen_uniform_sym_tiled", N, NB, seed, float(N if shift is None else shift), _ptr(tiles),
         _stream(stream))
    return tiles


def plgsy(tiles, N, NB, bump, seed, stream=None):
    call("gbx_dplgsy_tiled", N, NB, float(bump), seed, _ptr(tiles), _stream(stream))
    return tiles


class RefineInfo(ctypes.Structure):
    """gbx_refine_info of include/gbx_potrf.h."""
    _fields_ = [("iterations", ctypes.c_int), ("factor_retries", ctypes.c_int), ("shift", ctypes.c_double),
                ("backward_error", ctypes.c_double), ("anorm", ctypes.c_double),
                ("cond_estimate", ctypes.c_float), ("fp64_diag_tiles", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# Diagonal tiles whose condition estimate (max a_ii / min a_ii after their updates, a lower bound of
# the tile's condition number) exceeds this go to the FP64 POTRF route of the mixed factorisation:
# an FP32 Cholesky of a 512-tile can break down from about 1e4 on.
FP64_DIAG_COND = 1e4


def potrf_mixed(A_tiles, N, NB, prec="bf16", shift=0.0, W=None, work=None, stream=None, fp64_diag_cond=FP64_DIAG_COND,
                with_fp64_tiles=False):
    """Low-precision factorisation of an FP64 tile-major lower matrix into FP32 tiles W.
    Returns (W, work, status, cond_estimate) (and the number of diagonal tiles factorised in FP64
    with with_fp64_tiles=True)."""
    import torch
    need = _sz(0)
    call("gbx_potrf_mixed_bufferSize", N, NB, ctypes.byref(need))
    if W is None:
        W = torch.empty(A_tiles.numel(), dtype=torch.float32, device=A_tiles.device)
    if work is None or work.numel() < need.value:
        work = torch.empty(need.value, dtype=torch.uint8, device=A_tiles.device)
    s = _stream(stream)
    call("gbx_potrf_mixed", N, NB, _ptr(A_tiles), _ptr(W), PREC[prec], float(shift), float(fp64_diag_cond), _ptr(work),
         need.value, s)
    cond = ctypes.c_float(0)
    nf = ctypes.c_int(0)
    st = call("gbx_potrf_mixed_info", _ptr(work), N, NB, ctypes.byref(cond), ctypes.byref(nf), s)
    if with_fp64_tiles:
        return W, work, st, cond.value, nf.value
    return W, work, st, cond.value


def dposv_mixed(A_tiles, N, NB, B, prec="bf16", tol=1e-14, maxiter=200, stream=None, work=None, W=None,
                fp64_diag_cond=FP64_DIAG_COND):
    """Solves A X = B to FP64 backward error `tol` (B: (nrhs, N) CUDA float64, rows = right-hand
    sides). Returns (X, info dict, status)."""
    import torch
    nrhs = B.shape[0]
    need = _sz(0)
    call("gbx_dposv_mixed_bufferSize", N, NB, nrhs, ctypes.byref(need))
    if work is None or work.numel() < need.value:
        work = torch.empty(need.value, dtype=torch.uint8, device=A_tiles.device)
    if W is None:
        W = torch.empty(A_tiles.numel(), dtype=torch.float32, device=A_tiles.device)
    X = torch.empty_like(B)
    info = RefineInfo()
    st = lib().gbx_dposv_mixed(N, NB, _ptr(A_tiles), nrhs, _ptr(B), _ptr(X), PREC[prec], float(fp64_diag_cond),
                               float(tol), int(maxiter), _ptr(W), _ptr(work), need.value, ctypes.byref(info),
                               _stream(stream))
    if st < 0 and st != GBX_ERR_NOCONV:
        raise GbxError("gbx_dposv_mixed", st)
    return X, info.as_dict(), st


def backward_error_fp64(A_tiles, N, NB, B, X, stream=None):
    """Normwise backward error of each right-hand side, max_j ||b_j - A x_j||_inf / (||A||_inf
    ||x_j||_inf + ||b_j||_inf), from plain FP64 products over the lower tiles (gbx_dsymm_tiled), not
    from the solver's own double-float residual. B, X: (nrhs, N) CUDA float64, nrhs <= 16. Returns a
    list of nrhs floats."""
    import torch
    nrhs = B.shape[0]
    R = B.clone()
    call("gbx_dsymm_tiled", N, NB, _ptr(A_tiles), nrhs, -1.0, _ptr(X), 1.0, _ptr(R), _stream(stream))
    absA = A_tiles.abs()
    ones = torch.ones(1, N, dtype=torch.float64, device=A_tiles.device)
    rows = torch.zeros(1, N, dtype=torch.float64, device=A_tiles.device)
    call("gbx_dsymm_tiled", N, NB, _ptr(absA), 1, 1.0, _ptr(ones), 0.0, _ptr(rows), _stream(stream))
    anorm = rows.max()
    den = anorm * X.abs().amax(dim=1) + B.abs().amax(dim=1)
    return (R.abs().amax(dim=1) / den).tolist()


def split_f64(a, stream=None):
    """(hi, lo) FP32 tensors with hi + lo = a for an FP64 CUDA tensor (gbx_split_f64)."""
    import torch
    a = a.contiguous()
    hi = torch.empty(a.shape, dtype=torch.float32, device=a.device)
    lo = torch.empty(a.shape, dtype=torch.float32, device=a.device)
    call("gbx_split_f64", _ptr(a), _ptr(hi), _ptr(lo), a.numel(), _stream(stream))
    return hi, lo


def potri_tiled(tiles, N, NB, workspace=None, stream=None):
    """In place: the lower tiles of the factor L (from potrf_tiled) become the lower triangle of A^{-1}."""
    import torch
    need = _sz(0)
    call("gbx_dpotri_tiled_bufferSize", N, NB, ctypes.byref(need))
    if workspace is None or workspace.numel() < need.value:
        workspace = torch.empty(need.value, dtype=torch.uint8, device=tiles.device)
    call("gbx_dpotri_tiled", N, NB, _ptr(tiles), _ptr(workspace), need.value, _stream(stream))
    return tiles


def dposv_tiled_host(A_host, N, NB, B_host, tiles=None, X=None, work=None, L_host=None, X_host=None, stream=None,
                     check=True):
    """Factor + solve from host buffers with the copies overlapped (gbx_dposv_tiled_host).
    A_host: tile-major lower FP64 (pinned CPU tensor); B_host: (nrhs, N) pinned CPU tensor.
    Returns (L_host, X_host, status); with check=True the stream is synchronised first. A status > 0
    (first bad pivot) is returned whatever `check` says: the solve was skipped."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    nrhs = 1 if B_host.dim() == 1 else B_host.shape[0]
    need = _sz(0)
    call("gbx_dposv_tiled_host_bufferSize", N, NB, ctypes.byref(need))
    if work is None or work.numel() < need.value:
        work = torch.empty(need.value, dtype=torch.uint8, device=dev)
    tiles = torch.empty(A_host.numel(), dtype=torch.float64, device=dev) if tiles is None else tiles
    X = torch.empty(B_host.shape, dtype=torch.float64, device=dev) if X is None else X
    L_host = torch.empty(A_host.shape, dtype=torch.float64, pin_memory=True) if L_host is None else L_host
    X_host = torch.empty(B_host.shape, dtype=torch.float64, pin_memory=True) if X_host is None else X_host
    s = _stream(stream)
    st = call("gbx_dposv_tiled_host", N, NB, _ptr(A_host), _ptr(L_host), nrhs, _ptr(B_host), _ptr(X_host),
              _ptr(tiles), _ptr(X), _ptr(work), need.value, s)
    if st == 0:  # > 0: the factorisation stopped at that pivot and the solve was skipped
        st = call("gbx_dpotrf_tiled_status", _ptr(work), s) if check else None
    return L_host, X_host, st


def batched_tile_offsets(sizes, NB):
    """Element offset of every matrix's first tile slot in a concatenated tile-major batch, and the total."""
    import numpy as np
    nt = (np.asarray(sizes, dtype=np.int64) + NB - 1) // NB
    slots = nt * (nt + 1) // 2
    off = np.concatenate([[0], np.cumsum(slots)]) * NB * NB
    return off[:-1], int(off[-1])


def dposv_mixed_batched(A_tiles, sizes, NB, B, nrhs, prec="fp16", tol=1e-14, maxiter=200, stream=None, work=None,
                        W=None, fp64_diag_cond=FP64_DIAG_COND):
    """Batched mixed-precision solve. A_tiles: concatenated tile-major lower matrices (CUDA float64,
    batched_tile_offsets layout); B: concatenated column-major n_k x nrhs right-hand sides (CUDA
    float64). Returns (X, list of per-matrix info dicts, status)."""
    import numpy as np
    import torch
    n = np.ascontiguousarray(np.asarray(sizes, dtype=np.int32))
    batch = len(n)
    need = _sz(0)
    call("gbx_dposv_mixed_batched_bufferSize", batch, n.ctypes.data_as(ctypes.c_void_p), NB, nrhs,
         ctypes.byref(need))
    if work is None or work.numel() < need.value:
        work = torch.empty(need.value, dtype=torch.uint8, device=A_tiles.device)
    if W is None:
        W = torch.empty(A_tiles.numel(), dtype=torch.float32, device=A_tiles.device)
    X = torch.empty_like(B)
    infos = (RefineInfo * batch)()
    st = lib().gbx_dposv_mixed_batched(batch, n.ctypes.data_as(ctypes.c_void_p), NB, _ptr(A_tiles), nrhs, _ptr(B),
                                       _ptr(X), PREC[prec], float(fp64_diag_cond), float(tol), int(maxiter), _ptr(W),
                                       _ptr(work), need.value, ctypes.cast(infos, ctypes.c_void_p), _stream(stream))
    if st < 0 and st != GBX_ERR_NOCONV:
        raise GbxError("gbx_dposv_mixed_batched", st)
    return X, [i.as_dict() for i in infos], st


class MixedBatchedSolver:
    """The batched mixed-precision solve split as the C ABI offers it: the plan (task tables, once per
    batch shape; synchronises), the run (no host synchronisation, no allocation: capturable in a
    CUDA graph, e.g. torch.cuda.graph) and the result (synchronises). A, B, X, W: CUDA float64
    tensors laid out as for dposv_mixed_batched; X receives the solutions."""

    def __init__(self, sizes, NB, nrhs, prec="fp16", device=None, work=None, sched=0):
        import numpy as np
        import torch
        self.n = np.ascontiguousarray(np.asarray(sizes, dtype=np.int32))
        self.batch, self.NB, self.nrhs, self.prec = len(self.n), NB, nrhs, prec
        need = _sz(0)
        call("gbx_dposv_mixed_batched_bufferSize", self.batch, self._n(), NB, nrhs, ctypes.byref(need))
        self.work_bytes = need.value
        if work is None or work.numel() < need.value:
            work = torch.empty(need.value, dtype=torch.uint8, device=device)
        self.work = work
        call("gbx_dposv_mixed_batched_plan", self.batch, self._n(), NB, nrhs, PREC[prec], int(sched), _ptr(work),
             need.value, _stream(None))

    def _n(self):
        return self.n.ctypes.data_as(ctypes.c_void_p)

    def run(self, A_tiles, B, X, W, tol=1e-14, maxiter=200, fp64_diag_cond=FP64_DIAG_COND, stream=None):
        call("gbx_dposv_mixed_batched_exec", self.batch, self._n(), self.NB, _ptr(A_tiles), self.nrhs, _ptr(B), _ptr(X),
             PREC[self.prec], float(fp64_diag_cond), float(tol), int(maxiter), _ptr(W), _ptr(self.work),
             self.work_bytes, _stream(stream))

    def result(self, tol=1e-14, stream=None):
        infos = (RefineInfo * self.batch)()
        st = lib().gbx_dposv_mixed_batched_result(self.batch, self._n(), self.NB, self.nrhs, float(tol), _ptr(self.work),
                                                  ctypes.cast(infos, ctypes.c_void_p), _stream(stream))
        if st < 0 and st != GBX_ERR_NOCONV:
            raise GbxError("gbx_dposv_mixed_batched_result", st)
        return [i.as_dict() for i in infos], st


def gen_lowrank(tiles, N, NB, lam, U, V, G, stream=None):
    """Device generator of Q diag(lam) Q^T (see workloads.householder_factors)."""
    r = U.shape[1] if U is not None else 0
    Uc = U.T.contiguous() if r else None  # column-major N x r
    Vc = V.T.contiguous() if r else None
    Gc = G.T.contiguous() if r else None
    call("gbx_dgen_lowrank_sym_tiled", N, NB, _ptr(lam), _ptr(Uc) if r else None, _ptr(Vc) if r else None,
         _ptr(Gc) if r else None, r, _ptr(tiles), _stream(stream))
    return tiles


class Batch:
    """A packed batch of SPD systems on the device for gbx_dposv_batched.

    mats: list of (n_i x n_i) numpy float64 arrays (symmetric), or None together with `sizes` and
    `seed` to generate (M + M^T)/2 + n I on the device; rhs: list of (nrhs, n_i) arrays."""

    def __init__(self, mats, rhs, device, sizes=None, seed=42):
        import numpy as np
        import torch
        self.batch = len(mats) if mats is not None else len(sizes)
        self.nrhs = rhs[0].shape[0]
        n = np.array([m.shape[0] for m in mats] if mats is not None else list(sizes), dtype=np.int32)
        offA = np.zeros(self.batch, dtype=np.int64)
        offB = np.zeros(self.batch, dtype=np.int64)
        if self.batch > 1:
            offA[1:] = np.cumsum(n.astype(np.int64) ** 2)[:-1]
            offB[1:] = np.cumsum(n.astype(np.int64) * self.nrhs)[:-1]
        order = np.zeros(self.batch, dtype=np.int32)
        call("gbx_batched_order", self.batch, n.ctypes.data_as(_vp), order.ctypes.data_as(_vp))
        self.sizes = n
        to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
        self.n, self.offA, self.offB, self.order = to(n), to(offA), to(offB), to(order)
        total = int(np.sum(n.astype(np.int64) ** 2))
        if mats is not None:
            self.A0 = to(np.concatenate([np.asfortranarray(m).ravel(order="F") for m in mats]))
        else:
            self.A0 = torch.empty(total, dtype=torch.float64, device=device)
            call("gbx_dgen_uniform_sym_batched", self.batch, _ptr(self.n), _ptr(self.offA), seed, _ptr(self.A0),
                 _stream(None))
        Bh = np.concatenate([np.asarray(b, dtype=np.float64).reshape(self.nrhs, -1).ravel() for b in rhs])
        self.B0 = to(Bh)
        self.A, self.B = self.A0.clone(), self.B0.clone()
        self.L32 = torch.empty(total, dtype=torch.float32, device=device)
        self.info = torch.zeros(self.batch, dtype=torch.int32, device=device)
        self.work = torch.zeros(256, dtype=torch.uint8, device=device)
        self.flops = float(np.sum(n.astype(np.float64) ** 3) / 3.0)

    def reset(self):
        self.A.copy_(self.A0)
        self.B.copy_(self.B0)

    def set_order(self, order):
        """Replaces the queue order (a permutation of the matrix indices)."""
        import numpy as np
        import torch
        self.order = torch.from_numpy(np.ascontiguousarray(order, dtype=np.int32)).to(self.n.device)

    def solve(self, mode="fp64", refine=2, stream=None, ctas=0):
        """Launches the batched solve (asynchronous, capturable). mode: 'fp64' or 'fp32'."""
        call("gbx_dposv_batched_ex", self.batch, _ptr(self.n), _ptr(self.offA), _ptr(self.offB), _ptr(self.order),
             _ptr(self.A), _ptr(self.B), self.nrhs, 0 if mode == "fp64" else 1, int(refine), _ptr(self.L32),
             _ptr(self.info), int(ctas), _ptr(self.work), self.work.numel(), _stream(stream))

    def solutions(self):
        import numpy as np
        Bh = self.B.cpu().numpy()
        out, o = [], 0
        for ni in self.sizes:
            k = int(ni) * self.nrhs
            out.append(Bh[o:o + k].reshape(self.nrhs, int(ni)))
            o += k
        return out


TASK_NAMES = ["POTRF", "TRSM", "SYRK", "GEMM"] + ["?"] * 12  # record type = key >> 60
# (the mixed executor's POTRF records are its 128-block mini-tasks: sub-task = mini-task index)


def trace_records(buf):
    """Decodes a trace buffer (CUDA uint64 tensor given to gbx_set_trace_buffer) into dicts."""
    import numpy as np
    a = buf.cpu().numpy().view(np.uint64)
    n = min(int(a[0]), (len(a) - 2) // 4)
    rec = a[2:2 + 4 * n].reshape(n, 4)
    out = []
    for t0, t1, key, sc in rec:
        key, sc = int(key), int(sc)
        typ = key >> 60
        out.append({"start_ns": int(t0), "end_ns": int(t1), "type": TASK_NAMES[typ], "a": (key >> 40) & 0xFFFFF,
                    "b": (key >> 20) & 0xFFFFF, "c": key & 0xFFFFF, "sub": sc >> 32, "cta": sc & 0xFFFFFFFF})
    return out


def trace_to_chrome(records, path):
    """Writes records (trace_records) as Chrome trace JSON (one row per CTA)."""
    import json
    if not records:
        json.dump({"traceEvents": []}, open(path, "w"))
        return
    t0 = min(r["start_ns"] for r in records)
    ev = [{"name": "%s(%d,%d,%d)" % (r["type"], r["a"], r["b"], r["c"]), "cat": r["type"], "ph": "X",
           "ts": (r["start_ns"] - t0) / 1e3, "dur": (r["end_ns"] - r["start_ns"]) / 1e3, "pid": 0, "tid": r["cta"],
           "args": {"sub": r["sub"]}} for r in records]
    json.dump({"traceEvents": ev}, open(path, "w"))
