"""gal_integrate_noalloc: the integration entry point for callers that cannot
allocate device memory (plug-ins handed only their input and output buffers,
services that forbid allocation after start-up, hosts with a fixed device-memory
budget). It must give bitwise what gal_integrate gives with a caller
workspace, call after call, although every call reuses the same built-in
scratch array, and must refuse calls whose scratch would not fit.

Collected last on purpose (``zz``), so that a run that stops at the first
failure has run every other test first.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from galax_gb300.build import build

    build()
    import galax_gb300 as gx
    from galax_gb300 import _lib

    return gx, _lib, _lib.load()


def _batch(n, seed):
    from galax_gb300 import workloads as W
    from oracle import oracle as O

    return W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), n, seed=seed, tmax=400.0, smax=40)


def _device_inputs(b):
    import torch

    y0 = torch.as_tensor(b.y0, device="cuda").t().contiguous()
    t0 = torch.as_tensor(b.t0, device="cuda")
    t1 = torch.as_tensor(b.t1, device="cuda")
    offs = torch.as_tensor(b.save_offsets, device="cuda")
    ts = torch.as_tensor(b.save_ts, device="cuda")
    return y0, t0, t1, offs, ts


def _run(L, _lib, pot, cfg, inputs, n, *, noalloc):
    import torch

    y0, t0, t1, offs, ts = inputs
    total = ts.numel()
    out = torch.full((6, total), -1.0, dtype=torch.float64, device="cuda")
    status = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    steps = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    args = (pot.handle(), C.byref(cfg), y0.data_ptr(), t0.data_ptr(), t1.data_ptr(), offs.data_ptr(), ts.data_ptr(),
            total, out.data_ptr(), status.data_ptr(), steps.data_ptr(), None, n)
    if noalloc:
        rc = L.gal_integrate_noalloc(*args, stream)
        _lib.check(rc, "gal_integrate_noalloc")
    else:
        nb = C.c_size_t()
        _lib.check(L.gal_integrate_workspace_size(C.byref(cfg), n, C.byref(nb)), "workspace size")
        ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
        _lib.check(L.gal_integrate(*args, ws.data_ptr(), nb.value, stream), "gal_integrate")
    torch.cuda.synchronize()
    return out.cpu().numpy(), status.cpu().numpy(), steps.cpu().numpy()


@pytest.mark.parametrize("schedule", [True, False])
def test_noalloc_matches_workspace_path_on_consecutive_calls(env, schedule):
    gx, _lib, L = env
    mw = gx.MilkyWayPotential()
    integ = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                          max_steps=2**16, schedule=schedule)
    cfg = integ.config()
    # two different batches in a row: the second call must not see the first one's scratch
    for seed, n in ((11, 3000), (12, 1700)):
        b = _batch(n, seed)
        inputs = _device_inputs(b)
        ref = _run(L, _lib, mw, cfg, inputs, n, noalloc=False)
        got = _run(L, _lib, mw, cfg, inputs, n, noalloc=True)
        assert np.all(ref[1] == 0)
        np.testing.assert_array_equal(got[1], ref[1])
        np.testing.assert_array_equal(got[2], ref[2])
        # same kernels, same scratch layout: any difference, even one rounding,
        # would mean the shared array leaked state from the previous call
        np.testing.assert_array_equal(got[0], ref[0])


def test_noalloc_replays_from_a_cuda_graph(env):
    """Captured once into a CUDA graph (the use this entry point is made for),
    the two-pass schedule with its team fork/join replays to the workspace
    path's result bitwise, replay after replay."""
    import torch

    gx, _lib, L = env
    mw = gx.MilkyWayPotential()
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                        max_steps=2**16, schedule=True).config()
    n = 2500
    inputs = _device_inputs(_batch(n, 13))
    ref = _run(L, _lib, mw, cfg, inputs, n, noalloc=False)
    y0, t0, t1, offs, ts = inputs
    total = ts.numel()
    out = torch.empty((6, total), dtype=torch.float64, device="cuda")
    status = torch.empty((n,), dtype=torch.int32, device="cuda")
    steps = torch.empty((n,), dtype=torch.int64, device="cuda")

    def call(stream):
        return L.gal_integrate_noalloc(mw.handle(), C.byref(cfg), y0.data_ptr(), t0.data_ptr(), t1.data_ptr(),
                                       offs.data_ptr(), ts.data_ptr(), total, out.data_ptr(), status.data_ptr(),
                                       steps.data_ptr(), None, n, stream)

    _lib.check(call(torch.cuda.current_stream().cuda_stream), "gal_integrate_noalloc (eager)")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = call(torch.cuda.current_stream().cuda_stream)
    _lib.check(rc, "gal_integrate_noalloc (captured)")
    for _ in range(2):
        out.fill_(-1.0)
        status.fill_(-1)
        steps.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(status.cpu().numpy(), ref[1])
        np.testing.assert_array_equal(steps.cpu().numpy(), ref[2])
        np.testing.assert_array_equal(out.cpu().numpy(), ref[0])


def test_noalloc_rejects_calls_beyond_its_scratch(env):
    gx, _lib, L = env
    mw = gx.MilkyWayPotential()
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                        schedule=True).config()
    n = 40_000  # 136 bytes per orbit for the two-pass schedule: beyond 4 MiB
    nb = C.c_size_t()
    _lib.check(L.gal_integrate_workspace_size(C.byref(cfg), n, C.byref(nb)), "workspace size")
    assert nb.value > 4 * 1024 * 1024
    # rejected on the host before any device work, so no buffers are needed
    rc = L.gal_integrate_noalloc(mw.handle(), C.byref(cfg), None, None, None, None, None, 0, None, None, None,
                                 None, n, None)
    assert rc == 5  # GAL_ERR_TOO_LARGE
    assert b"built-in array holds 4194304" in L.gal_last_error()
