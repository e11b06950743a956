"""The TTG-compatible C++ API (include/ttg.h) and its runtime.

CPU: host-task semantics; the reference's own potrf flowgraph (examples/potrf/potrf.h, plgsy.h,
result.h) and unmodified driver (testing_dpotrf.cc) compiled against include/ttg.h — run when a
reference checkout is present — and checked bit for bit against the oracle's restatement.
GPU: the device-task contract (the scenarios of tests/unit/device_coro.cc) and this project's
device-branch potrf flowgraph (ttg_gb300/potrf) against the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
from oracle import build as obuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "ttg_cpp")
OUT = os.path.join(CPP, "_build")
CUDA_INC = "/usr/local/cuda/include"
CUDA_LIB = "/usr/local/cuda/lib64"


def _build(src, exe, nvcc=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, exe)
    if os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(src), *[os.path.getmtime(os.path.join(ROOT, "include", "ttg", f))
                                     for f in ("tt.h", "runtime.h", "buffer.h", "device/task.h")]):
        return out
    if nvcc:
        cmd = ["nvcc", "-std=c++20", "-gencode", "arch=compute_103a,code=sm_103a", "-O1", "-I",
               os.path.join(ROOT, "include"), src, "-o", out, *extra]
    else:
        cmd = ["g++", "-std=c++20", "-O1", "-pthread", "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC, src, "-o",
               out, *extra, "-L" + CUDA_LIB, "-lcudart"]
    subprocess.check_call(cmd)
    return out


def _run(cmd, timeout=600):
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout + r.stderr


def test_host_task_semantics():
    exe = _build(os.path.join(CPP, "host_tt.cc"), "host_tt")
    rc, out = _run([exe], timeout=120)
    assert rc == 0 and "ALL PASS" in out, out


def test_abort_is_opt_in_process_termination():
    """ttg::abort() throws by default; with set_abort_terminates(true) (the reference-faithful mode)
    it ends the process with SIGABRT, as the reference's abort on a non-SPD pivot does."""
    import signal
    exe = _build(os.path.join(CPP, "host_tt.cc"), "host_tt")
    rc, out = _run([exe, "abort"], timeout=120)
    assert rc == -signal.SIGABRT, (rc, out)
    assert "PASS abort-throws" in out and "ttg::abort() called" in out and "ALL PASS" not in out


def _ref_bins():
    bins = obuild.build_ref_flowgraph()
    if bins is None:
        pytest.skip("no reference checkout: the reference flowgraph cannot be compiled here")
    return bins


@pytest.mark.parametrize("N,NB", [(160, 32), (100, 32), (1000, 128), (257, 64)])
def test_reference_flowgraph_on_this_runtime_matches_oracle(tmp_path, N, NB):
    ref_potrf, _ = _ref_bins()
    out = str(tmp_path / "f.bin")
    rc, log = _run([ref_potrf, str(N), str(NB), out], timeout=300)
    assert rc == 0, log
    got = np.fromfile(out)
    t = oracle.plgsy_tiles(N, NB, N, 3872)
    st, _, _ = oracle.potrf_tiled(t, N, NB, nthreads=4)
    assert st == 0
    assert np.array_equal(got, t)  # same tile kernels, same per-tile update order: same bits


def test_reference_driver_unmodified_passes_its_check():
    _, drv = _ref_bins()
    rc, out = _run([drv, "-N", "1000", "-t", "128"], timeout=300)
    assert rc == 0 and "Factorization is CORRECT" in out, out


@pytest.mark.gpu
def test_device_task_contract(gbx, cuda):
    exe = _build(os.path.join(CPP, "device_coro.cu"), "device_coro", nvcc=True)
    rc, out = _run([exe], timeout=300)
    assert rc == 0 and "ALL PASS" in out, out


def _driver(gbx):
    from ttg_gb300 import build as gb
    return gb.build_driver()


@pytest.mark.gpu
@pytest.mark.parametrize("queue", [False, True], ids=["per-task-launch", "device-queue"])
@pytest.mark.parametrize("N,NB", [(1000, 128), (2048, 512), (160, 32)])
def test_gb300_potrf_flowgraph_matches_oracle(gbx, cuda, tmp_path, N, NB, queue):
    """The potrf flowgraph's device tasks, launched one by one or recorded into the device task queue
    (one persistent launch per batch), give the oracle's factor."""
    drv = _driver(gbx)
    out = str(tmp_path / "L.bin")
    rc, log = _run([drv, "-N", str(N), "-t", str(NB), "-o", out] + (["-q"] if queue else []), timeout=600)
    assert rc == 0 and "Factorization is CORRECT" in log, log
    got = np.fromfile(out)
    ref = oracle.plgsy_tiles(N, NB, N, 3872)
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0)[0] == 0
    L, Lref = oracle.tiles_to_lower(got, N, NB), oracle.tiles_to_lower(ref, N, NB)
    assert np.max(np.abs(L - Lref)) <= 1e-12 * np.max(np.abs(Lref))


@pytest.mark.gpu
def test_gb300_potrf_flowgraph_timed_iterations(gbx, cuda):
    drv = _driver(gbx)
    rc, log = _run([drv, "-N", "4096", "-t", "512", "-n", "2", "-x"], timeout=600)
    assert rc == 0, log
    assert log.count("TTG Execution Time") == 2, log


@pytest.mark.gpu
@pytest.mark.parametrize("N,NB,nrhs,queue", [(1000, 128, 3, False), (2500, 512, 1, False), (160, 32, 16, False),
                                            (1000, 128, 3, True), (2500, 512, 2, True)])
def test_gb300_potrs_flowgraph_matches_oracle(gbx, cuda, tmp_path, N, NB, nrhs, queue):
    """The solve as a TTG flowgraph (forward and backward TRSM/GEMM device tasks over right-hand-side
    tiles, ttg_gb300/potrf/potrs.h) after the factorisation flowgraph: the driver's backward-error
    check passes and X equals the oracle's solve with the same factor."""
    drv = _driver(gbx)
    lf, xf = str(tmp_path / "L.bin"), str(tmp_path / "X.bin")
    rc, log = _run([drv, "-N", str(N), "-t", str(NB), "-s", str(nrhs), "-o", lf, "-p", xf] + (["-q"] if queue else []),
                   timeout=600)
    assert rc == 0 and "Factorization is CORRECT" in log and "Solve is CORRECT" in log, log
    L = np.fromfile(lf)
    X = np.fromfile(xf).reshape(nrhs, N)
    i = np.arange(N)[:, None]
    r = np.arange(nrhs)[None, :]
    B = ((7919 * i + 104729 * r) % 1000) / 500.0 - 1.0  # the driver's right-hand sides, N x nrhs
    Xref = oracle.potrs_tiled(L, N, NB, B)
    assert np.max(np.abs(X.T - Xref)) <= 1e-12 * np.max(np.abs(Xref))


@pytest.mark.gpu
def test_chain_of_device_tasks_through_the_device_queue(gbx, cuda):
    """A chain of device tasks (keys only, and one device buffer travelling the chain) completes with
    the device task queue: each task's sends run right after its recording, and the runtime's idle
    and fence triggers run what was recorded."""
    from ttg_gb300 import build as gb
    chain = gb.build_chain()
    for flows in ("0", "1"):
        rc, log = _run([chain, "-f", flows, "-n", "2000", "-q"], timeout=300)
        assert rc == 0 and "avg" in log, log
