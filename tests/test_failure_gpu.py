"""Failure paths on the GPU, made without faulting it.

* A bounded device wait that runs out: gu_check_grid_barrier launches the grid
  barrier every persistent kernel is built on with one CTA that never arrives
  (a barrier nothing completes); the others give up after the given limit and
  the call returns GU_ERR_TIMEOUT.  The device stays usable: a graph handle made
  before it passes a parity search afterwards.
* Out of memory: gu_debug_fail_allocations makes the library's next device or
  pinned allocations fail on the host side; each call reports
  GU_ERR_OUT_OF_MEMORY, and the same handle works once the failures are spent.
* The timing and device-choice entry points (util_device.cu:4-76 in the
  reference) return what they promise.

The reference has no error statuses: checkCudaErrors exits the process
(util_device.cuh:10-22).
"""
import ctypes

import numpy as np
import pytest

import gu
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

L = gu.lib()
L.gu_set_wait_limit.argtypes = [ctypes.c_double]
L.gu_get_wait_limit.argtypes = [ctypes.POINTER(ctypes.c_double)]
L.gu_check_grid_barrier.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
L.gu_debug_fail_allocations.argtypes = [ctypes.c_int64, ctypes.c_int64]


def _bfs_matches_oracle(g, hg, srcs):
    s = torch.as_tensor(srcs, device="cuda")
    d = torch.empty((len(srcs), hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, d, variant="auto")
    torch.cuda.synchronize()
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    np.testing.assert_array_equal(d.cpu().numpy(), ref)


def test_grid_barrier_wait_runs_out_and_device_stays_usable():
    hg = gu.HostGraph.rmat(13, 16, seed=5)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 300, seed=1)
    _bfs_matches_oracle(g, hg, srcs)
    t = ctypes.c_double()
    assert L.gu_check_grid_barrier(-1, 1.0, None, ctypes.byref(t)) == gu.OK, L.gu_last_error()
    assert 0 < t.value < 0.5
    # CTA 3 never arrives: the others' wait ends by its 2 ms limit, not by a hang
    st = L.gu_check_grid_barrier(3, 0.002, None, ctypes.byref(t))
    assert st == 6, (st, L.gu_last_error())  # GU_ERR_TIMEOUT
    msg = L.gu_last_error()
    assert b"block 3 never arrived" in msg and b"0 of" in msg
    assert 0.002 <= t.value < 0.5
    # the context and the handle made before are still usable
    _bfs_matches_oracle(g, hg, srcs)
    assert L.gu_check_grid_barrier(-1, 1.0, None, ctypes.byref(t)) == gu.OK
    assert L.gu_check_grid_barrier(10 ** 6, 1.0, None, ctypes.byref(t)) == 1
    g.close()


def test_wait_limit_is_a_launch_setting():
    v = ctypes.c_double()
    assert L.gu_get_wait_limit(ctypes.byref(v)) == gu.OK and v.value == pytest.approx(4.0)
    try:
        assert L.gu_set_wait_limit(0.5) == gu.OK
        assert L.gu_get_wait_limit(ctypes.byref(v)) == gu.OK and v.value == pytest.approx(0.5)
        hg = gu.HostGraph.rmat(14, 16, seed=2)
        g = gu.Graph(hg)
        _bfs_matches_oracle(g, hg, gu.sources(hg.n, 200, seed=3))  # every level ends well within 0.5 s
        bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
        srcs = gu.sources(hg.n, 64, seed=4)
        g.bc(torch.as_tensor(srcs, device="cuda"), bc)
        want = oracle.bc(hg.R, hg.C, hg.n, srcs, nthreads=8)
        np.testing.assert_allclose(bc.cpu().numpy(), want, rtol=1e-12, atol=1e-300)
        g.close()
    finally:
        assert L.gu_set_wait_limit(4.0) == gu.OK


def test_out_of_memory_paths_leave_handles_usable():
    hg = gu.HostGraph.rmat(13, 16, seed=7)
    srcs = gu.sources(hg.n, 300, seed=2)
    try:
        # graph creation: the second allocation (C) fails, nothing is kept
        free0 = torch.cuda.mem_get_info()[0]
        assert L.gu_debug_fail_allocations(1, 1) == gu.OK
        with pytest.raises(gu.GuError) as e:
            gu.Graph(hg)
        assert e.value.status == 3
        assert torch.cuda.mem_get_info()[0] >= free0 - (8 << 20)
        g = gu.Graph(hg)
        # the batched search's workspace (both of its tries fail)
        assert L.gu_debug_fail_allocations(0, 2) == gu.OK
        s = torch.as_tensor(srcs, device="cuda")
        d = torch.empty((len(srcs), hg.n), dtype=torch.int32, device="cuda")
        with pytest.raises(gu.GuError) as e:
            g.bfs(s, d, variant="warp")
        assert e.value.status == 3
        _bfs_matches_oracle(g, hg, srcs)
        # the host-buffer form's device staging (both of its tries fail)
        assert L.gu_debug_fail_allocations(0, 2) == gu.OK
        with pytest.raises(gu.GuError) as e:
            g.bfs_host(srcs, "auto")
        assert e.value.status == 3
        np.testing.assert_array_equal(g.bfs_host(srcs, "auto"), oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, 8)[0])
        # BC: a fresh handle, its workspace and work items not yet built
        g2 = gu.Graph(hg)
        bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
        assert L.gu_debug_fail_allocations(0, 1) == gu.OK
        with pytest.raises(gu.GuError) as e:
            g2.bc(s[:64], bc)
        assert e.value.status == 3
        assert L.gu_debug_fail_allocations(0, 0) == gu.OK
        g2.bc(s[:64], bc)
        want = oracle.bc(hg.R, hg.C, hg.n, srcs[:64], nthreads=8)
        np.testing.assert_allclose(bc.cpu().numpy(), want, rtol=1e-12, atol=1e-300)
        g.close()
        g2.close()
    finally:
        L.gu_debug_fail_allocations(0, 0)


def test_timer_and_choose_device():
    chosen = ctypes.c_int(-5)
    assert L.gu_choose_device(0, ctypes.byref(chosen)) == gu.OK and chosen.value == 0
    assert L.gu_choose_device(-1, ctypes.byref(chosen)) == gu.OK
    assert 0 <= chosen.value < torch.cuda.device_count()
    assert L.gu_choose_device(torch.cuda.device_count(), ctypes.byref(chosen)) == 1
    assert L.gu_choose_device(-2, ctypes.byref(chosen)) == 1
    L.gu_choose_device(0, ctypes.byref(chosen))
    hg = gu.HostGraph.rmat(14, 16, seed=1)
    g = gu.Graph(hg)
    s = torch.as_tensor(gu.sources(hg.n, 256, seed=1), device="cuda")
    d = torch.empty((256, hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, d)
    t = ctypes.c_void_p()
    assert L.gu_timer_start(None, ctypes.byref(t)) == gu.OK
    for _ in range(5):
        g.bfs(s, d)
    sec = ctypes.c_double(-1)
    assert L.gu_timer_stop(t, None, ctypes.byref(sec)) == gu.OK
    kernel = g.last_launch()[0]
    assert 5 * kernel * 0.9 <= sec.value < 5.0
    assert L.gu_timer_start(None, None) == 1
    assert L.gu_timer_stop(None, None, ctypes.byref(sec)) == 1
    g.close()
