"""Failure detection on the GPU without a GPU fault: a device wait that
nothing satisfies gives up after its time limit and reports a status (the
context stays usable); injected allocation failures come back as
GG_ERR_NOMEM and the library recovers on the next call (context and server).
Nothing here traps, faults or hangs the GPU."""
import ctypes
import time

import numpy as np
import pytest

import gpugrid as gg
import oracle as O
import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _small_job(seed=0, N=128, S=8, n=3000):
    uv, vals = synth.uniform(n, 4, N - 4, seed=seed)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    return N, S, uv, vals, gcf


def _check_grid(ctx, opts, N, S, uv, vals, gcf):
    out = torch.empty(N * N, dtype=torch.complex64, device="cuda")
    ctx.grid(opts, out, torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(), N, S)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(N, N)
    pairs = lambda c: np.stack([np.asarray(c).reshape(-1).real,
                                np.asarray(c).reshape(-1).imag], -1).astype(np.float64)
    ref = O.grid_pz(uv, pairs(vals), pairs(gcf), N, S)
    err = max(np.abs(got.real - ref[0, 0]).max(), np.abs(got.imag - ref[1, 0]).max())
    assert err <= 1e-6 * np.abs(ref).max()


OPTS = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, layout=gg.LAYOUT_INTERLEAVED)


def test_device_wait_gives_up_and_context_stays_usable():
    with gg.Context(0) as ctx:
        s = torch.cuda.current_stream()
        t0 = time.perf_counter()
        st = gg.LIB.gg_selftest_wait_timeout(ctx._h, ctypes.c_void_p(s.cuda_stream))
        dt = time.perf_counter() - t0
        assert st == gg.ERR_TIMEOUT, gg.LIB.gg_last_error()
        assert 0.3 <= dt < 30.0
        assert ctx.read_flags() == [0, 0, 0, 0]   # the self-test clears its flag
        _check_grid(ctx, OPTS, *_small_job(1))
        assert ctx.read_flags() == [0, 0, 0, 0]


def test_injected_allocation_failure_then_recovery():
    with gg.Context(0) as ctx:                   # fresh: its workspace is empty
        N, S, uv, vals, gcf = _small_job(2)
        assert gg.LIB.gg_debug_inject_alloc_failures(1) == gg.OK
        out = torch.empty(N * N, dtype=torch.complex64, device="cuda")
        with pytest.raises(gg.GridError) as e:
            ctx.grid(OPTS, out, torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
                     torch.from_numpy(gcf.reshape(-1)).cuda(), N, S)
        assert e.value.code == gg.ERR_NOMEM and "injected" in str(e.value)
        _check_grid(ctx, OPTS, N, S, uv, vals, gcf)   # the next call allocates and works
    gg.LIB.gg_debug_inject_alloc_failures(0)


def test_server_request_fails_cleanly_on_allocation_failure():
    N, S, uv, vals, gcf = _small_job(3)
    with gg.Server(streams=1, options=OPTS) as srv:
        gid = srv.add_gcf(gcf)
        outs = [np.zeros(N * N, np.complex64) for _ in range(4)]
        req = lambda o: gg.Server.request(uv.ctypes.data, vals.ctypes.data, o.ctypes.data,
                                          len(uv), N, S, gid)
        assert gg.LIB.gg_debug_inject_alloc_failures(1) == gg.OK
        t = srv.submit(req(outs[0]))
        with pytest.raises(gg.GridError) as e:
            srv.wait(t, timeout=30)
        assert e.value.code == gg.ERR_NOMEM
        srv.release(t)
        gg.LIB.gg_debug_inject_alloc_failures(0)
        tickets = [srv.submit(req(o)) for o in outs[1:]]
        for t in tickets:
            assert srv.wait(t, timeout=30).status == 0
            srv.release(t)
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 3 and st["hbm_in_use"] == 0
    pairs = lambda c: np.stack([c.reshape(-1).real, c.reshape(-1).imag], -1).astype(np.float64)
    ref = O.grid_pz(uv, pairs(vals), pairs(gcf), N, S)
    for o in outs[1:]:
        g = o.reshape(N, N)
        err = max(np.abs(g.real - ref[0, 0]).max(), np.abs(g.imag - ref[1, 0]).max())
        assert err <= 1e-6 * np.abs(ref).max()
