"""lbmx_moment_sums_noalloc: the FP64 mass / momentum sums computed without
any device allocation, for callers that may not call cudaMalloc where they
need the sums (a stall-free stepping loop, a framework that owns all device
memory through its own pool, a process under a hard memory cap).

The entry point reads the caller's density and velocity fields and keeps its
partial sums in a fixed array inside the library.  Its results must match the
sums lbmx_moments returns for the same step (computed by the step kernel with
its own scratch buffer), call after call, and an FP64 sum of the same values
at sizes below one block, ragged sizes and sizes where the grid is capped and
each thread reads several nodes.  This file is collected last so a failure
here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

# FP64 sums of the same FP32 values in a different order
RTOL = 1e-12


def _noalloc(L, rho_dev, u_dev, out_ptr, stream=None):
    return L.lib.lbmx_moment_sums_noalloc(rho_dev.data_ptr(), u_dev.data_ptr(), rho_dev.numel(), out_ptr, stream)


def _host_call(L, rho, u):
    out = (ctypes.c_double * 3)()
    assert _noalloc(L, rho, u, ctypes.addressof(out)) == 0
    return np.array(list(out))


@pytest.mark.parametrize("nx,ny", [(512, 384), (1024, 512)])
def test_noalloc_sums_match_step_sums_on_consecutive_calls(nx, ny):
    import torch

    # 1024 x 512 = 524,288 nodes: more than the 1024 blocks x 256 threads the
    # reduction launches, so the grid-stride loop runs
    c = C.random_state(C.cavity_moving_wall(nx, ny, op=C.MRT, nu=0.05), seed=21)
    L = C.make_lattice(c)
    n = L.n
    rho = torch.empty(n, dtype=torch.float32, device="cuda")
    u = torch.empty(2 * n, dtype=torch.float32, device="cuda")
    for steps in (7, 6):  # two rounds: the shared scratch is reused
        L.step(steps)
        ref = (ctypes.c_double * 3)()
        L._check(L.lib.lbmx_moments(L.h, rho.data_ptr(), u.data_ptr(), ref))
        ref = np.array(list(ref))
        torch.cuda.synchronize()
        first = _host_call(L, rho, u)
        second = _host_call(L, rho, u)
        assert np.allclose(first, ref, rtol=RTOL, atol=1e-9 * abs(ref[0])), (first, ref)
        assert np.array_equal(first, second)  # deterministic block order
        # result delivered to device memory on a caller stream: the call does
        # not block, the sums are there once the stream has run it
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            dev_out = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
        assert _noalloc(L, rho, u, dev_out.data_ptr(), s.cuda_stream) == 0
        s.synchronize()
        assert np.array_equal(dev_out.cpu().numpy(), first)


@pytest.mark.parametrize("n", [1, 100, 1000, 262_145, 3_000_001])
def test_noalloc_sums_of_ragged_sizes(n):
    """Sizes below one block, not a multiple of 256, and above the capped
    grid, against an FP64 sum of the same FP32 values, on two calls."""
    import torch

    L = C.make_lattice(C.taylor_green(16, 16))
    g = np.random.default_rng(n)
    rho_h = (1.0 + 0.05 * g.standard_normal(n)).astype(np.float32)
    u_h = (0.1 * g.standard_normal(2 * n)).astype(np.float32)
    r64 = rho_h.astype(np.float64)
    want = np.array([r64.sum(), (r64 * u_h[:n]).sum(), (r64 * u_h[n:]).sum()])
    rho = torch.from_numpy(rho_h).cuda()
    u = torch.from_numpy(u_h).cuda()
    torch.cuda.synchronize()
    first = _host_call(L, rho, u)
    second = _host_call(L, rho, u)
    assert np.allclose(first, want, rtol=RTOL, atol=1e-12 * n), (first, want)
    assert np.array_equal(first, second)


def test_noalloc_rejects_bad_sizes():
    import torch

    c = C.taylor_green(16, 16)
    L = C.make_lattice(c)
    rho = torch.ones(256, dtype=torch.float32, device="cuda")
    u = torch.zeros(512, dtype=torch.float32, device="cuda")
    out = (ctypes.c_double * 3)()
    assert L.lib.lbmx_moment_sums_noalloc(rho.data_ptr(), u.data_ptr(), 0, ctypes.addressof(out), None) == 1
    too_big = 2 ** 31
    assert L.lib.lbmx_moment_sums_noalloc(rho.data_ptr(), u.data_ptr(), too_big, ctypes.addressof(out), None) == 8


def test_noalloc_call_captured_in_a_cuda_graph():
    """With its sums going to device memory the call never synchronises, so
    it can be captured into a CUDA graph (after a first call outside any
    capture, which resolves the library's scratch array); every replay
    writes the sums of the fields' values at that time."""
    import torch

    c = C.taylor_green(64, 32)
    L = C.make_lattice(c)
    n = 256 * 128
    rng = np.random.default_rng(3)
    rho = torch.from_numpy(rng.uniform(0.9, 1.1, n).astype(np.float32)).cuda()
    u = torch.from_numpy(rng.normal(0.0, 0.05, 2 * n).astype(np.float32)).cuda()
    first = _host_call(L, rho, u)
    out = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        assert _noalloc(L, rho, u, out.data_ptr(), s.cuda_stream) == 0
    g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), first)
    rho.mul_(1.5)
    u.mul_(-2.0)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), _host_call(L, rho, u))
