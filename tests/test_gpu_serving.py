"""GPU tests of the batched and served forms, through the C ABI.

* batched plans: a plan launched directly, and the same plan captured into a
  CUDA graph and replayed, match per-job gridding;
* the server: every request's grid is the same gridded alone (one job per
  call) and gridded in the mix of a continuously batched stream, within the
  FP32-compensated tolerance (1e-6 normwise); admission by HBM budget,
  rejection, cancellation, wait timeouts, resident grids and arrival traces.
No test here faults or hangs the GPU: every failure is made on the host.
"""
import time

import numpy as np
import pytest

import gpugrid as gg
import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 1e-6


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = gg.Context(0)
    yield c
    c.close()


def make_request_data(k, rng):
    N = int(rng.choice([64, 128, 256, 512]))
    S = int(rng.choice([8, 16]))
    n = int(rng.integers(200, 20000))
    uv, vals = synth.tracks(N, nant=16, ntime=max(4, n // 120 + 1), npts=n, seed=k)
    return N, S, uv, vals


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def grid_alone(ctx, opts, N, S, uv, vals, gcf):
    out = torch.empty(N * N, dtype=torch.complex64, device="cuda")
    ctx.grid(opts, out, torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(), N, S)
    torch.cuda.synchronize()
    return out.cpu().numpy()


GCF = {S: synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64) for S in (8, 16)}
OPTS = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, layout=gg.LAYOUT_INTERLEAVED)


def test_plan_and_cuda_graph_replay(ctx):
    rng = np.random.default_rng(1)
    jobs, keep, want = [], [], []
    for k in range(6):
        N, S, uv, vals = make_request_data(k, rng)
        d = [torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(GCF[S].reshape(-1)).cuda(),
             torch.full((N * N,), float("nan"), dtype=torch.complex64, device="cuda")]
        keep.append((N, d))
        jobs.append(gg.Context.make_job(d[3], d[0], d[1], d[2], N, S))
        want.append(grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S]))
    plan = gg.Plan(ctx, OPTS, jobs)
    plan.launch()
    torch.cuda.synchronize()
    for (N, d), w in zip(keep, want):
        assert relerr(d[3].cpu().numpy(), w) <= TOL
    # capture the launch in a CUDA graph, clear the outputs, replay twice
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan.launch(s)  # warm-up on the capture stream
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.launch(s)
    for _ in range(2):
        for _, d in keep:
            d[3].fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        for (N, d), w in zip(keep, want):
            assert relerr(d[3].cpu().numpy(), w) <= TOL
    assert plan.read_flags() == [0, 0, 0, 0]
    plan.close()


def test_server_results_same_alone_and_in_mix(ctx):
    rng = np.random.default_rng(2)
    data = [make_request_data(100 + k, rng) for k in range(24)]
    with gg.Server(streams=2, options=OPTS) as srv:
        gids = {S: srv.add_gcf(GCF[S]) for S in (8, 16)}
        outs, tickets, keep = [], [], []
        for N, S, uv, vals in data:
            uvp = np.ascontiguousarray(uv)
            vp = np.ascontiguousarray(vals)
            out = np.full(N * N, np.nan, np.complex64)
            keep.append((uvp, vp))
            outs.append(out)
            tickets.append(srv.submit(gg.Server.request(
                uvp.ctypes.data, vp.ctypes.data, out.ctypes.data, len(uv), N, S, gids[S])))
        for t in tickets:
            r = srv.wait(t, timeout=60)
            assert r.status == 0 and r.latency_s > 0
            srv.release(t)
        st = srv.stats()
        assert st["completed"] == len(data) and st["failed"] == 0
        assert st["batches"] >= 1 and st["p99_latency_s"] >= st["p50_latency_s"] > 0
        assert st["hbm_in_use"] == 0
    for (N, S, uv, vals), out in zip(data, outs):
        assert relerr(out, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL


def test_server_device_inputs_resident_grids_and_budget(ctx):
    rng = np.random.default_rng(3)
    data = [make_request_data(200 + k, rng) for k in range(10)]
    grid_bytes = max(N * N * 8 for N, _, _, _ in data)
    # a budget for about two requests at a time: admission must serialise
    budget = 3 * grid_bytes + 3 * 20000 * 64 + 2 * 4096 * 16 + 65536
    with gg.Server(streams=3, hbm_budget=budget, options=OPTS) as srv:
        gids = {S: srv.add_gcf(GCF[S]) for S in (8, 16)}
        tickets, keep = [], []
        for N, S, uv, vals in data:
            d_uv, d_v = torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda()
            keep.append((d_uv, d_v))
            tickets.append(srv.submit(gg.Server.request(
                d_uv.data_ptr(), d_v.data_ptr(), None, len(uv), N, S, gids[S],
                flags=gg.REQ_INPUTS_ON_DEVICE | gg.REQ_KEEP_RESIDENT)))
        for t, (N, S, uv, vals) in zip(tickets, data):
            r = srv.wait(t, timeout=60)
            assert r.status == 0 and r.device_out
            host = np.empty(N * N, np.complex64)
            _copy_device_to_host(r.device_out, host)
            assert relerr(host, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL
            srv.release(t)
        st = srv.stats()
        assert st["completed"] == len(data)
        assert st["hbm_peak"] <= budget
        assert st["hbm_in_use"] == 0
        # a request larger than the whole budget is refused at submission
        N = 4096
        big = gg.Server.request(keep[0][0].data_ptr(), keep[0][1].data_ptr(), None, 1000,
                                N, 8, gids[8], flags=gg.REQ_INPUTS_ON_DEVICE | gg.REQ_KEEP_RESIDENT)
        with pytest.raises(gg.GridError) as e:
            srv.submit(big)
        assert e.value.code == gg.ERR_BUDGET
        assert srv.stats()["rejected"] == 1


def _copy_device_to_host(dev_ptr, host):
    """cudaMemcpy (device to host) of a raw device pointer, through the CUDA
    runtime libgg.so is linked against (already loaded: found by soname)."""
    import ctypes
    f = ctypes.CDLL("libcudart.so.13").cudaMemcpy
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    f.restype = ctypes.c_int
    assert f(host.ctypes.data, ctypes.c_void_p(dev_ptr), host.nbytes, 2) == 0


def test_server_trace_cancel_timeout(ctx):
    rng = np.random.default_rng(4)
    data = [make_request_data(300 + k, rng) for k in range(40)]
    with gg.Server(streams=2, options=OPTS) as srv:
        gids = {S: srv.add_gcf(GCF[S]) for S in (8, 16)}
        keep, reqs = [], []
        for N, S, uv, vals in data:
            out = np.zeros(N * N, np.complex64)
            keep.append((uv, vals, out))
            reqs.append(gg.Server.request(uv.ctypes.data, vals.ctypes.data, out.ctypes.data,
                                          len(uv), N, S, gids[S]))
        # Poisson arrivals over ~0.2 s, plus one far in the future
        offs = np.cumsum(rng.exponential(0.005, len(reqs)))
        offs[-1] = 30.0
        tickets = srv.submit_schedule(reqs, offs)
        with pytest.raises(gg.GridError) as e:
            srv.wait(int(tickets[-1]), timeout=0.05)
        assert e.value.code == gg.ERR_TIMEOUT
        srv.cancel(int(tickets[-1]))
        with pytest.raises(gg.GridError) as e:
            srv.wait(int(tickets[-1]), timeout=1)
        assert e.value.code == gg.ERR_CANCELLED
        for t in tickets[:-1]:
            assert srv.wait(int(t), timeout=60).status == 0
        srv.drain(timeout=60)
        st = srv.stats()
        assert st["completed"] == len(reqs) - 1 and st["cancelled"] == 1
    for (N, S, uv, vals), (_, _, out) in zip(data[:-1], keep[:-1]):
        assert relerr(out, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL


def test_server_times_autotune_trials_only_while_young(ctx):
    """With autotune 1 the server times trials only during its first
    GG_SERVER_TUNE_BATCHES batches: a support class first seen later takes
    the cached or default configuration (autotune 2) and is not timed, so no
    trial lands on a request's latency under load.  Results stay correct."""
    rng = np.random.default_rng(5)
    gg.autotune_clear()
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED, autotune=1)
    with gg.Server(streams=1, options=o) as srv:
        gids = {S: srv.add_gcf(GCF[S]) for S in (8, 16)}

        def one(S, seed):
            N = 256
            uv, vals = synth.tracks(N, nant=16, ntime=40, npts=4000, seed=seed)
            out = np.full(N * N, np.nan, np.complex64)
            t = srv.submit(gg.Server.request(uv.ctypes.data, vals.ctypes.data, out.ctypes.data,
                                             len(uv), N, S, gids[S]))
            assert srv.wait(t, timeout=60).status == 0
            srv.release(t)
            assert relerr(out, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL

        one(8, 500)                    # first batch: support 8 is tuned
        assert "support 8 " in gg.autotune_report()
        for k in range(gg.SERVER_TUNE_BATCHES):
            one(8, 501 + k)            # one request per batch
        assert srv.stats()["batches"] > gg.SERVER_TUNE_BATCHES
        one(16, 600)                   # after the window: not timed
        assert "support 16 " not in gg.autotune_report()
    gg.autotune_clear()


def test_autotune_lookup_only_never_times(ctx):
    """autotune 2 reuses the cache and, with nothing cached, runs the
    default configuration without trials."""
    gg.autotune_clear()
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED, autotune=2)
    N, S = 512, 16
    uv, vals = synth.tracks(N, nant=24, ntime=400, npts=None, seed=77)
    got = grid_alone(ctx, o, N, S, uv, vals, GCF[S])
    assert gg.autotune_report().strip() == ""
    assert relerr(got, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL


def test_server_pipeline_keeps_flags_with_their_batch(ctx):
    """The server pipelines batches (input copies, kernels on a slot, output
    copies on a shared stream) and gives every batch in flight its own device
    flag words.  Twelve host requests, one per batch, submitted at once over
    two slots: a flag raised on the first three batches (from the host,
    behind their kernels) reaches exactly those requests while later batches
    run on the same slots, and every grid equals the request gridded alone."""
    rng = np.random.default_rng(8)
    data = [make_request_data(800 + k, rng) for k in range(12)]
    with gg.Server(streams=2, max_batch_jobs=1, options=OPTS) as srv:
        gids = {S: srv.add_gcf(GCF[S]) for S in (8, 16)}
        outs, reqs = [], []
        for N, S, uv, vals in data:
            outs.append(np.full(N * N, np.nan, np.complex64))
            reqs.append(gg.Server.request(uv.ctypes.data, vals.ctypes.data,
                                          outs[-1].ctypes.data, len(uv), N, S, gids[S]))
        gg.inject_device_flags(gg.DEVFLAG_INDEX, 3)
        try:
            tickets = srv.submit_schedule(reqs, np.zeros(len(reqs)))
            res = [srv.wait(int(t), timeout=120) for t in tickets]
        finally:
            gg.inject_device_flags(0, 0)
        for t in tickets:
            srv.release(int(t))
        assert [r.device_flags for r in res] == [gg.DEVFLAG_INDEX] * 3 + [0] * 9
        assert all(r.status == gg.OK for r in res)
        for (N, S, uv, vals), out in zip(data, outs):
            assert relerr(out, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL
        st = srv.stats()
        assert st["completed"] == 12 and st["batches"] == 12 and st["hbm_in_use"] == 0


def test_server_reports_device_flags(ctx):
    """Device-side failures reach the requests of their batch: the server
    reads the batch's flag words back behind its kernels.  A bounded-wait
    timeout (raised from the host by a one-thread kernel, no real wait) fails
    the batch's requests with GG_ERR_TIMEOUT; dropped visibilities are
    reported and the request succeeds; input declared tile-sorted that is
    not (a real device detection) fails with GG_ERR_UNSORTED.  Requests of
    later batches are unaffected."""
    rng = np.random.default_rng(6)
    data = [make_request_data(600 + k, rng) for k in range(3)]
    with gg.Server(streams=1, options=OPTS) as srv:
        gids = {S: srv.add_gcf(GCF[S]) for S in (8, 16)}

        def one(k, inject=0, check=True):
            N, S, uv, vals = data[k]
            out = np.full(N * N, np.nan, np.complex64)
            gg.inject_device_flags(inject, 1 if inject else 0)
            try:
                t = srv.submit(gg.Server.request(uv.ctypes.data, vals.ctypes.data,
                                                 out.ctypes.data, len(uv), N, S, gids[S]))
                r = srv.wait(t, timeout=60, check=check)
            finally:
                gg.inject_device_flags(0, 0)
            srv.release(t)
            return r, out

        r, _ = one(0, gg.DEVFLAG_TIMEOUT, check=False)
        assert r.status == gg.ERR_TIMEOUT and r.device_flags == gg.DEVFLAG_TIMEOUT
        r, out = one(1, gg.DEVFLAG_INDEX)
        assert r.status == gg.OK and r.device_flags == gg.DEVFLAG_INDEX
        N, S, uv, vals = data[1]
        assert relerr(out, grid_alone(ctx, OPTS, N, S, uv, vals, GCF[S])) <= TOL
        r, out = one(2)
        assert r.status == gg.OK and r.device_flags == 0
        st = srv.stats()
        assert st["completed"] == 2 and st["failed"] == 1 and st["hbm_in_use"] == 0
    srt = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                     layout=gg.LAYOUT_INTERLEAVED, input_sorted=True)
    with gg.Server(streams=1, options=srt) as srv:
        N, S = 256, 8
        uv, vals = synth.uniform(5000, 8, N - 8, seed=61)   # not tile-sorted
        gid = srv.add_gcf(GCF[S])
        out = np.zeros(N * N, np.complex64)
        t = srv.submit(gg.Server.request(uv.ctypes.data, vals.ctypes.data, out.ctypes.data,
                                         len(uv), N, S, gid))
        r = srv.wait(t, timeout=60, check=False)
        assert r.status == gg.ERR_UNSORTED and r.device_flags & gg.DEVFLAG_UNSORTED
        srv.release(t)
        order = synth.tile_sort(uv, N, 32, S)
        uv2, v2 = np.ascontiguousarray(uv[order]), np.ascontiguousarray(vals[order])
        t = srv.submit(gg.Server.request(uv2.ctypes.data, v2.ctypes.data, out.ctypes.data,
                                         len(uv2), N, S, gid))
        assert srv.wait(t, timeout=60).device_flags == 0
        srv.release(t)
