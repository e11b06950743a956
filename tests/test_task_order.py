"""The task orders of the persistent executors (CPU, through the C ABI's host-side decode):
gbx_dpotrf_tiled's block order and the mixed factorisation's tile order. Each must list every
task of the right-looking tiled Cholesky exactly once, and every task's predecessors before it,
which is what lets CTAs take tasks in order and wait on their predecessors without deadlock:
  POTRF(k)     after SYRK(j, k) for all j < k   (every update of the diagonal block)
  TRSM(m, k)   after POTRF(k) and GEMM(m, k, j) for all j < k
  SYRK(k, n)   after TRSM(n, k) and SYRK(k-1, n)
  GEMM(m,n,k)  after TRSM(m, k), TRSM(n, k) and GEMM(m, n, k-1)
"""
import ctypes

import numpy as np
import pytest

POTRF, TRSM, SYRK, GEMM = 0, 1, 2, 3


def _order(gbx, fn, nt):
    key = np.zeros(4, dtype=np.int32)
    n = gbx.call(fn, nt, -1, None)
    out = []
    for t in range(n):
        gbx.call(fn, nt, t, key.ctypes.data_as(ctypes.c_void_p))
        out.append(tuple(int(v) for v in key))
    return out


SPLIT = 4  # the block executor runs TRSM(K+1,K) (on the critical path) as 4 row sub-tasks


def _parts(fn, m, k):
    return SPLIT if fn != "gbx_mixed_task" and m == k + 1 else 1


def _expected(nt, fn="gbx_dag_task"):
    tasks = set()
    for k in range(nt):
        tasks.add((POTRF, k, 0, 0))
        for m in range(k + 1, nt):
            for s in range(_parts(fn, m, k)):
                tasks.add((TRSM, m, k, s))
            tasks.add((SYRK, k, m, 0))
            for n in range(k + 1, m):
                tasks.add((GEMM, m, n, k))
    return tasks


def _trsm(fn, m, k):
    return [(TRSM, m, k, s) for s in range(_parts(fn, m, k))]


def _deps(task, fn="gbx_dag_task"):
    ty, a, b, c = task
    if ty == POTRF:
        return [(SYRK, j, a, 0) for j in range(a)]
    if ty == TRSM:
        return [(POTRF, b, 0, 0)] + [(GEMM, a, b, j) for j in range(b)]
    if ty == SYRK:
        return _trsm(fn, b, a) + ([(SYRK, a - 1, b, 0)] if a > 0 else [])
    return _trsm(fn, a, c) + _trsm(fn, b, c) + ([(GEMM, a, b, c - 1)] if c > 0 else [])


@pytest.mark.parametrize("fn", ["gbx_dag_task", "gbx_mixed_task"])
@pytest.mark.parametrize("nt", [1, 2, 3, 5, 8, 17, 33])
def test_order_is_complete_and_topological(gbx, fn, nt):
    order = _order(gbx, fn, nt)
    assert len(order) == len(set(order)), "a task appears twice"
    assert set(order) == _expected(nt, fn)
    pos = {t: i for i, t in enumerate(order)}
    for t, i in pos.items():
        for d in _deps(t, fn):
            assert pos[d] < i, (t, d)


@pytest.mark.parametrize("fn", ["gbx_dag_task", "gbx_mixed_task"])
def test_order_argument_checks(gbx, fn):
    L = gbx.lib()
    key = (ctypes.c_int * 4)()
    assert getattr(L, fn)(0, -1, None) == gbx.GBX_ERR_ARG
    n = getattr(L, fn)(4, -1, None)
    assert n == len(_expected(4, fn))
    assert getattr(L, fn)(4, n, key) == gbx.GBX_ERR_ARG
    assert getattr(L, fn)(4, 0, None) == gbx.GBX_ERR_ARG


@pytest.mark.parametrize("lead", [1, 3, 40, 10**9])
@pytest.mark.parametrize("nt", [2, 5, 17, 33])
def test_order_with_trailing_lead_is_complete_and_topological(gbx, nt, lead):
    """The emulated executor's order: `lead` trailing tasks of each step ahead of its TRSMs."""
    key = np.zeros(4, dtype=np.int32)
    n = gbx.call("gbx_dag_task_lead", nt, lead, -1, None)
    order = []
    for t in range(n):
        gbx.call("gbx_dag_task_lead", nt, lead, t, key.ctypes.data_as(ctypes.c_void_p))
        order.append(tuple(int(v) for v in key))
    assert len(order) == len(set(order)) and set(order) == _expected(nt)
    pos = {t: i for i, t in enumerate(order)}
    for t, i in pos.items():
        for d in _deps(t):
            assert pos[d] < i, (t, d)
    if nt >= 5 and lead < 10**9:  # the leading trailing tasks really precede the step's TRSMs
        k0 = [i for i, t in enumerate(order) if t == (TRSM, 2, 1, 0)][0]
        assert order[k0 - 1][0] in (SYRK, GEMM)


def test_dag_lead_setting(gbx):
    L = gbx.lib()
    assert L.gbx_set_dag_lead(-2) == gbx.GBX_ERR_ARG
    assert L.gbx_dag_task_lead(4, -1, -1, None) == gbx.GBX_ERR_ARG
    assert L.gbx_set_dag_lead(100) == 0 and L.gbx_set_dag_lead(-1) == 0
