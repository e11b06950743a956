"""CPU tests of the C-ABI boundary: the library loads, exports every symbol its header declares,
and validates arguments without touching a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(gbx_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ["gbx_dpotrf_tile", "gbx_dtrsm_rlt_tile", "gbx_dsyrk_ln_tile", "gbx_dgemm_nt_tile",
              "gbx_dpotrf_tiled", "gbx_dpotrs_tiled"]:
        assert n in names


def test_library_exports_every_declared_symbol(gbx):
    L = gbx.lib()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_python_signatures_cover_header(gbx):
    assert declared_symbols() <= set(gbx.SIGNATURES)


def test_built_for_sm103a(gbx):
    assert gbx.lib().gbx_built_arch() == 1030


def test_argument_validation_without_gpu(gbx):
    L = gbx.lib()
    sz = ctypes.c_size_t(0)
    assert L.gbx_dpotrf_tiled_bufferSize(-1, 32, ctypes.byref(sz)) == gbx.GBX_ERR_ARG
    assert L.gbx_dpotrf_tiled_bufferSize(1000, 200, ctypes.byref(sz)) == gbx.GBX_ERR_ARG  # 200: no block edge
    assert L.gbx_dpotrf_tiled_bufferSize(32768, 512, ctypes.byref(sz)) == 0
    ntb = 32768 // 128
    assert sz.value >= 64 + ntb * (ntb + 1) // 2 * 4
    assert L.gbx_dpotrf_tiled(100, 0, None, None, 0, None) == gbx.GBX_ERR_ARG
    assert L.gbx_dgemm_nt_tile(10, 10, 10, None, 5, None, 10, None, 10, None) == gbx.GBX_ERR_ARG
    assert L.gbx_dtrsm_rlt_tile(10, 10, None, 10, None, 5, None) == gbx.GBX_ERR_ARG
    assert L.gbx_dpotrs_tiled(100, 32, None, 1, None, 50, None) == gbx.GBX_ERR_ARG
    # split: negative count, missing pointers; an empty split does nothing
    assert L.gbx_split_f64(None, None, None, -1, None) == gbx.GBX_ERR_ARG
    assert L.gbx_split_f64(None, None, None, 8, None) == gbx.GBX_ERR_ARG
    assert L.gbx_split_f64(None, None, None, 0, None) == 0
    # mixed solvers: operand precision 0 (bf16), 1 (fp16) or 2 (fp8 e4m3); NB 256 or 512
    dummy = ctypes.c_void_p(16)
    assert L.gbx_potrf_mixed(1000, 256, dummy, dummy, 3, ctypes.c_double(0.0), ctypes.c_double(1e4), dummy, 1 << 30,
                             None) == \
        gbx.GBX_ERR_ARG
    assert L.gbx_potrf_mixed(1000, 768, dummy, dummy, 0, ctypes.c_double(0.0), ctypes.c_double(1e4), dummy, 1 << 30,
                             None) == \
        gbx.GBX_ERR_ARG
    assert L.gbx_potrf_mixed_bufferSize(1000, 1024, ctypes.byref(sz)) == gbx.GBX_ERR_ARG


def test_dag_block_edge_setting(gbx):
    """The executor's block edge: 0 (automatic), 32, 64 or 128; anything else is refused. The
    workspace follows the edge (64-blocks for small N by default: four times the counters)."""
    L = gbx.lib()
    for bad in (-1, 16, 96, 256):
        assert L.gbx_set_dag_block_edge(bad) == gbx.GBX_ERR_ARG
    a, b = ctypes.c_size_t(0), ctypes.c_size_t(0)
    try:
        assert L.gbx_set_dag_block_edge(128) == 0
        assert L.gbx_dpotrf_tiled_bufferSize(2048, 128, ctypes.byref(a)) == 0
        assert L.gbx_set_dag_block_edge(64) == 0
        assert L.gbx_dpotrf_tiled_bufferSize(2048, 128, ctypes.byref(b)) == 0
        assert b.value > a.value
    finally:
        assert L.gbx_set_dag_block_edge(0) == 0


@pytest.mark.parametrize("mode,N,edge", [(0, 4096, 64), (0, 4608, 128), (1, 2048, 64), (1, 2560, 128),
                                         (1, 4096, 128)])
def test_automatic_block_edge_follows_update_mode(gbx, mode, N, edge):
    """64-blocks up to N = 4096 with FP64 FMA updates, up to N = 2048 with the tensor-core updates:
    the automatic workspace equals the one of the forced edge."""
    L = gbx.lib()
    a, b = ctypes.c_size_t(0), ctypes.c_size_t(0)
    try:
        assert L.gbx_set_fp64_update(mode) == 0
        assert L.gbx_set_dag_block_edge(0) == 0
        assert L.gbx_dpotrf_tiled_bufferSize(N, 512, ctypes.byref(a)) == 0
        assert L.gbx_set_dag_block_edge(edge) == 0
        assert L.gbx_dpotrf_tiled_bufferSize(N, 512, ctypes.byref(b)) == 0
        assert a.value == b.value
    finally:
        L.gbx_set_dag_block_edge(0)
        L.gbx_set_fp64_update(0)


def test_wait_timeout_setting(gbx):
    L = gbx.lib()
    old = L.gbx_get_wait_timeout_ns()
    L.gbx_set_wait_timeout_ns(12345)
    assert L.gbx_get_wait_timeout_ns() == 12345
    L.gbx_set_wait_timeout_ns(old)


def test_batched_mixed_workspace_without_gpu(gbx):
    L = gbx.lib()
    n = (ctypes.c_int * 3)(700, 256, 1300)
    sz, one = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert L.gbx_dposv_mixed_batched_bufferSize(0, n, 256, 2, ctypes.byref(sz)) == gbx.GBX_ERR_ARG
    assert L.gbx_dposv_mixed_batched_bufferSize(3, n, 200, 2, ctypes.byref(sz)) == gbx.GBX_ERR_ARG
    assert L.gbx_dposv_mixed_batched_bufferSize(3, n, 1024, 2, ctypes.byref(sz)) == gbx.GBX_ERR_ARG  # NB 256 or 512
    assert L.gbx_dposv_mixed_batched_bufferSize(3, n, 256, 17, ctypes.byref(sz)) == gbx.GBX_ERR_ARG
    bad = (ctypes.c_int * 2)(100, 0)
    assert L.gbx_potrf_mixed_batched_bufferSize(2, bad, 256, ctypes.byref(sz)) == gbx.GBX_ERR_ARG
    assert L.gbx_dposv_mixed_batched_bufferSize(3, n, 256, 2, ctypes.byref(sz)) == 0
    slots = sum((k + 255) // 256 * ((k + 255) // 256 + 1) // 2 for k in (700, 256, 1300))
    assert sz.value > slots * 256 * 256 * 2  # at least the low-precision copies
    assert L.gbx_dposv_mixed_bufferSize(700, 256, 2, ctypes.byref(one)) == 0
    assert 0 < one.value < sz.value


def test_batched_mixed_plan_exec_result_argument_checks(gbx):
    """The split batched solve rejects bad arguments before any device work (no GPU needed)."""
    L = gbx.lib()
    n = (ctypes.c_int * 2)(700, 300)
    dummy = ctypes.c_void_p(16)
    d = ctypes.c_double
    assert L.gbx_dposv_mixed_batched_plan(2, n, 200, 2, 0, 0, dummy, 1 << 40, None) == gbx.GBX_ERR_ARG
    assert L.gbx_dposv_mixed_batched_plan(2, n, 256, 2, 3, 0, dummy, 1 << 40, None) == gbx.GBX_ERR_ARG
    assert L.gbx_dposv_mixed_batched_plan(2, n, 256, 2, 0, 2, dummy, 1 << 40, None) == gbx.GBX_ERR_ARG  # schedule
    assert L.gbx_dposv_mixed_batched_plan(2, n, 256, 2, 0, 0, dummy, 16, None) == gbx.GBX_ERR_WORKSPACE
    ex = L.gbx_dposv_mixed_batched_exec
    assert ex(2, n, 256, dummy, 2, dummy, dummy, 0, d(1e4), d(0.0), 10, dummy, dummy, 1 << 40, None) == \
        gbx.GBX_ERR_ARG  # tolerance must be positive
    assert ex(2, n, 256, dummy, 2, dummy, dummy, 0, d(-1.0), d(1e-14), 10, dummy, dummy, 1 << 40, None) == \
        gbx.GBX_ERR_ARG  # FP64-route threshold must be >= 0
    assert ex(2, n, 256, None, 2, dummy, dummy, 0, d(1e4), d(1e-14), 10, dummy, dummy, 1 << 40, None) == \
        gbx.GBX_ERR_ARG
    assert ex(2, n, 256, dummy, 2, dummy, dummy, 0, d(1e4), d(1e-14), 10, dummy, dummy, 16, None) == \
        gbx.GBX_ERR_WORKSPACE
    assert L.gbx_dposv_mixed_batched_result(2, n, 256, 2, d(1e-14), None, None, None) == gbx.GBX_ERR_ARG
    assert L.gbx_potrf_mixed(1000, 256, dummy, dummy, 0, d(0.0), d(-1.0), dummy, 1 << 30, None) == gbx.GBX_ERR_ARG
