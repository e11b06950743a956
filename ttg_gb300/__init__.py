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

_ERRNAMES = {GBX_ERR_ARG: "invalid argument", GBX_ERR_CUDA: "CUDA runtime error",
             GBX_ERR_TIMEOUT: "device-side wait timed out", GBX_ERR_WORKSPACE: "workspace too small"}

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
    "gbx_get_wait_timeout_ns": (_u64, []),
    "gbx_dpotrf_tile_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_dpotrf_tile": (_i, [_i, _vp, _i, _vp, _sz, _vp, _vp]),
    "gbx_dtrsm_rlt_tile": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dsyrk_ln_tile": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dgemm_nt_tile": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dpotrf_tiled_bufferSize": (_i, [_i, _i, _szp]),
    "gbx_dpotrf_tiled": (_i, [_i, _i, _vp, _vp, _sz, _vp]),
    "gbx_dpotrf_tiled_status": (_i, [_vp, _vp]),
    "gbx_dpotrs_tiled": (_i, [_i, _i, _vp, _i, _vp, _i, _vp]),
    "gbx_dplgsy_tiled": (_i, [_i, _i, _d, _ull, _vp, _vp]),
    "gbx_dgen_uniform_sym_tiled": (_i, [_i, _i, _ull, _d, _vp, _vp]),
    "gbx_dplgsy_tile": (_i, [_d, _i, _i, _vp, _i, _i, _i, _i, _ull, _vp]),
    "gbx_dag_timeout_selftest": (_i, [_i, _vp, _vp, _sz, _u64, _vp]),
    "gbx_gemm_bf16_nt_f32": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _vp]),
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
