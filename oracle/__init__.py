"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Imported by the tests, by `__graft_entry__.smoke()` (for the expected result) and by the CPU-baseline
leg of `bench.py`. The product path never imports this package.
"""
import ctypes
import glob
import os

import numpy as np

from . import build as _build

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_ip = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_tile_slot.restype = ctypes.c_int64
        L.orc_tile_slot.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_tiles_from_colmajor.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int64, _dp]
        L.orc_tiles_to_colmajor.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int64]
        L.orc_plgsy_tile.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong]
        L.orc_plgsy_tiles.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong, _dp]
        L.orc_uniform_elem.restype = ctypes.c_double
        L.orc_uniform_elem.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64]
        L.orc_gen_uniform_sym_tiles.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_double, _dp]
        L.orc_gen_uniform_sym_colmajor.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_double, _dp,
                                                   ctypes.c_int64]
        L.orc_potrf_tile.restype = ctypes.c_int
        L.orc_potrf_tile.argtypes = [ctypes.c_int, _dp, ctypes.c_int]
        L.orc_trsm_rlt_tile.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int]
        L.orc_syrk_ln_tile.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int]
        L.orc_gemm_nt_tile.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp,
                                       ctypes.c_int, _dp, ctypes.c_int]
        L.orc_trsm_rln_tile.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int]
        L.orc_gemm_nn_tile.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp,
                                       ctypes.c_int, _dp, ctypes.c_int]
        L.orc_blas_load.restype = ctypes.c_int
        L.orc_blas_load.argtypes = [ctypes.c_char_p]
        L.orc_blas_loaded.restype = ctypes.c_int
        L.orc_potrf_tiled.restype = ctypes.c_int
        L.orc_potrf_tiled.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, _ip,
                                      _i64p, ctypes.c_int64, _i64p]
        L.orc_priority.restype = ctypes.c_int64
        L.orc_priority.argtypes = [ctypes.c_int] * 5
        L.orc_potrs_tiled.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int64]
        L.orc_check_dpotrf.restype = ctypes.c_double
        L.orc_check_dpotrf.argtypes = [ctypes.c_int, _dp, _dp]
        L.orc_frob_residual.restype = ctypes.c_double
        L.orc_frob_residual.argtypes = [ctypes.c_int, _dp, _dp]
        L.orc_dposv_batched.argtypes = [ctypes.c_int, _ip, _i64p, _i64p, _dp, _dp, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, _ip]
        L.orc_gen_uniform_sym_batched.argtypes = [ctypes.c_int, _ip, _i64p, ctypes.c_uint64, _dp]
        L.orc_potri_tiled.restype = ctypes.c_int
        L.orc_potri_tiled.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def ntiles(N, NB):
    return (N + NB - 1) // NB


def nslots(N, NB):
    nt = ntiles(N, NB)
    return nt * (nt + 1) // 2


def alloc_tiles(N, NB):
    return np.zeros(nslots(N, NB) * NB * NB, dtype=np.float64)


def tile_slot(m, n, NT):
    return n * NT - n * (n - 1) // 2 + (m - n)


def tiles_from_full(A, NB):
    """Full symmetric (or lower) N x N matrix -> lower tiles (flat float64)."""
    N = A.shape[0]
    Af = np.asfortranarray(A, dtype=np.float64)
    t = alloc_tiles(N, NB)
    lib().orc_tiles_from_colmajor(N, NB, _p(Af), N, _p(t))
    return t


def tiles_to_lower(tiles, N, NB):
    """Lower tiles -> N x N lower-triangular matrix (upper zero)."""
    A = np.zeros((N, N), dtype=np.float64, order="F")
    lib().orc_tiles_to_colmajor(N, NB, _p(tiles), _p(A), N)
    return np.ascontiguousarray(A)


def plgsy_tiles(N, NB, bump, seed):
    t = alloc_tiles(N, NB)
    lib().orc_plgsy_tiles(N, NB, float(bump), seed, _p(t))
    return t


def uniform_sym_tiles(N, NB, seed=42, shift=None):
    t = alloc_tiles(N, NB)
    lib().orc_gen_uniform_sym_tiles(N, NB, seed, float(N if shift is None else shift), _p(t))
    return t


def uniform_sym_full(N, seed=42, shift=None):
    A = np.zeros((N, N), dtype=np.float64, order="F")
    lib().orc_gen_uniform_sym_colmajor(N, seed, float(N if shift is None else shift), _p(A), N)
    return np.ascontiguousarray(A)


def find_openblas():
    """Path of the OpenBLAS shared library bundled with scipy (or numpy), or None."""
    pats = []
    try:
        import scipy
        d = os.path.dirname(os.path.dirname(scipy.__file__))
        pats.append(os.path.join(d, "scipy.libs", "libscipy_openblas-*.so"))
        pats.append(os.path.join(d, "scipy.libs", "libopenblas*.so"))
    except ImportError:
        pass
    for p in pats:
        hits = sorted(glob.glob(p))
        if hits:
            return hits[0]
    return None


def load_openblas():
    path = find_openblas()
    if path is None:
        return False
    return lib().orc_blas_load(path.encode()) == 0


def potrf_tiled(tiles, N, NB, nthreads=0, use_blas=False, trace=False):
    """Runs the restated flowgraph in place. Returns (status, tile_info, trace_list)."""
    info = ctypes.c_int(0)
    ntr = ctypes.c_int64(0)
    nt = ntiles(N, NB)
    cap = nt + nt * (nt - 1) + nt * (nt - 1) * (nt - 2) // 6 if trace else 0
    tr = np.zeros(max(cap, 1), dtype=np.int64)
    st = lib().orc_potrf_tiled(N, NB, _p(tiles), nthreads, 1 if use_blas else 0, ctypes.byref(info),
                               tr.ctypes.data_as(_i64p) if trace else None, cap, ctypes.byref(ntr))
    return st, info.value, (tr[: min(ntr.value, cap)] if trace else None)


def potrs_tiled(tiles, N, NB, B):
    X = np.asfortranarray(np.array(B, dtype=np.float64).reshape(N, -1))
    lib().orc_potrs_tiled(N, NB, _p(tiles), X.shape[1], _p(X), N)
    return X


def check_dpotrf(L, A0):
    N = A0.shape[0]
    Lf = np.asfortranarray(L, dtype=np.float64)
    Af = np.asfortranarray(A0, dtype=np.float64)
    return lib().orc_check_dpotrf(N, _p(Lf), _p(Af))


def frob_residual(L, A0):
    N = A0.shape[0]
    Lf = np.asfortranarray(L, dtype=np.float64)
    Af = np.asfortranarray(A0, dtype=np.float64)
    return lib().orc_frob_residual(N, _p(Lf), _p(Af))


def batched_offsets(sizes, nrhs=1):
    n = np.asarray(sizes, dtype=np.int32)
    offA = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)]).astype(np.int64)
    offB = np.concatenate([[0], np.cumsum(n.astype(np.int64) * nrhs)]).astype(np.int64)
    return n, offA, offB


def gen_uniform_sym_batched(sizes, seed=42):
    """All matrices of the batched generator, concatenated column-major (offsets from batched_offsets)."""
    n, offA, _ = batched_offsets(sizes)
    A = np.empty(int(offA[-1]), dtype=np.float64)
    lib().orc_gen_uniform_sym_batched(len(n), n.ctypes.data_as(_ip), offA.ctypes.data_as(_i64p), seed, _p(A))
    return A


def dposv_batched(sizes, A, B, nrhs=1, nthreads=0, use_blas=False):
    """In place: A (concatenated column-major matrices) := factors, B := solutions. Returns info array."""
    n, offA, offB = batched_offsets(sizes, nrhs)
    assert A.dtype == np.float64 and A.flags.c_contiguous and A.size >= offA[-1]
    assert B.dtype == np.float64 and B.flags.c_contiguous and B.size >= offB[-1]
    info = np.zeros(len(n), dtype=np.int32)
    lib().orc_dposv_batched(len(n), n.ctypes.data_as(_ip), offA.ctypes.data_as(_i64p), offB.ctypes.data_as(_i64p),
                            _p(A), _p(B), nrhs, nthreads, 1 if use_blas else 0, info.ctypes.data_as(_ip))
    return info


def potri_tiled(tiles, N, NB):
    """In place: the lower tiles of L become the lower triangle of A^{-1} (restated TRTRI + LAUUM)."""
    return lib().orc_potri_tiled(N, NB, _p(tiles))
