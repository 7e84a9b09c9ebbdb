"""The request loop: jobs of different sizes and parameters submitted together, admitted by HBM footprint
and overlapping on the GPU, give byte-identical partition files, bounds and labels to the same jobs run
alone through the plain job API; a failing request reports its error without disturbing the others."""
import numpy as np
import pytest

from metapart_gb300 import native, serve, synth

pytestmark = pytest.mark.gpu

# (workload, reads, k, scans, threads, chunks, min3, interleaved)
JOBS = [
    ("plain_small", 30000, 27, 1, 2, 4, False, False),
    ("plain_large", 60000, 31, 2, 4, 8, False, False),
    ("hotspot", 30000, 25, 1, 2, 4, False, False),
    ("plain_small", 8000, 21, 1, 2, 4, True, False),
    ("interleaved_small", 20000, 27, 2, 2, 4, False, True),
    ("plain_large", 120000, 29, 3, 4, 8, False, False),
    ("plain_small", 2000, 31, 1, 1, 2, False, False),
    ("min3", 20000, 31, 1, 2, 4, True, False),
]


def _alone(ctx, data, k, scans, threads, chunks, min3, il):
    job, bounds, _ = native.run_pipeline(ctx, data, k, chunks, scans, threads, min3=min3, interleaved=il)
    try:
        out, sizes = job.output()
        return bytes(out), sizes.copy(), bounds.copy(), job.labels()
    finally:
        job.close()


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def test_results_same_alone_and_in_the_mix(ctx):
    import torch
    datas = [synth.fastq_bytes(synth.workload(w, n, seed=100 + i)) for i, (w, n, *_) in enumerate(JOBS)]
    want = [_alone(ctx, d, *spec[2:]) for d, spec in zip(datas, JOBS)]
    ins = [torch.frombuffer(bytearray(d), dtype=torch.uint8).pin_memory() for d in datas]
    outs = [torch.empty(len(d) * (2 if spec[7] else 1) + 64, dtype=torch.uint8).pin_memory()
            for d, spec in zip(datas, JOBS)]
    sizes = [np.zeros(16 * spec[4], dtype=np.uint64) for spec in JOBS]
    labels = [np.zeros(len(w[3]), dtype=np.uint32) for w in want]
    params = [serve.RequestParams(k, int(m3), s, t, c, int(il)) for (_, _, k, s, t, c, m3, il) in JOBS]
    fps = [serve.footprint(i.data_ptr(), i.numel(), p) for i, p in zip(ins, params)]
    # a budget that holds the two largest requests at once but not all of them
    budget = sum(sorted(fps)[-2:])
    with serve.Server(ctx, slots=4, hbm_budget=budget) as srv:
        tickets = [srv.submit(i.data_ptr(), i.numel(), p, o.data_ptr(), o.numel(), fs, lb)
                   for i, p, o, fs, lb in zip(ins, params, outs, sizes, labels)]
        res = [srv.result(t) for t in tickets]
        st = srv.stats()
    for r, (w_out, w_sizes, w_bounds, w_labels), o, fs, lb, spec in zip(res, want, outs, sizes, labels, JOBS):
        assert r.status == 0, (spec, r.error)
        assert r.out_total == len(w_out)
        assert bytes(o[:r.out_total].numpy()) == w_out, spec
        assert np.array_equal(fs, w_sizes), spec
        assert np.array_equal(np.array(r.bounds, dtype=np.uint64), w_bounds), spec
        assert np.array_equal(lb, w_labels), spec
        assert r.t_submit_ms <= r.t_admit_ms <= r.t_done_ms
    assert st["completed"] == len(JOBS)
    assert st["peak_running"] >= 2            # jobs overlapped
    assert st["peak_reserved"] <= budget      # admission kept the reservations inside the budget
    assert st["reserved"] == 0 and st["running"] == 0


def test_failing_request_reports_and_others_finish(ctx):
    import torch
    good = synth.fastq_bytes(synth.workload("plain_small", 4000, seed=5))
    w_out, _, w_bounds, _ = _alone(ctx, good, 27, 1, 2, 4, False, False)
    gi = torch.frombuffer(bytearray(good), dtype=torch.uint8).pin_memory()
    go = torch.empty(len(good) + 64, dtype=torch.uint8).pin_memory()
    bad_out = torch.empty(len(good) + 64, dtype=torch.uint8).pin_memory()
    small_out = torch.empty(16, dtype=torch.uint8).pin_memory()
    with serve.Server(ctx, slots=2) as srv:
        t_bad = srv.submit(gi.data_ptr(), gi.numel(), serve.RequestParams(40, 0, 1, 2, 4, 0), bad_out.data_ptr(),
                           bad_out.numel())
        t_small = srv.submit(gi.data_ptr(), gi.numel(), serve.RequestParams(27, 0, 1, 2, 4, 0), small_out.data_ptr(),
                             small_out.numel())
        t_good = srv.submit(gi.data_ptr(), gi.numel(), serve.RequestParams(27, 0, 1, 2, 4, 0), go.data_ptr(),
                            go.numel())
        r_bad, r_small, r_good = srv.result(t_bad), srv.result(t_small), srv.result(t_good)
    assert r_bad.status == native_code("MP_EARG") and "k must be" in r_bad.error
    assert r_small.status == native_code("MP_EARG") and "too small" in r_small.error
    assert r_good.status == 0
    assert bytes(go[:r_good.out_total].numpy()) == w_out
    assert np.array_equal(np.array(r_good.bounds, dtype=np.uint64), w_bounds)


def test_released_or_unknown_ticket_is_refused(ctx):
    """A result is released once: polling its ticket again (blocking or not), or a ticket never issued,
    returns MP_EARG instead of waiting for a result that will not come."""
    import torch
    data = synth.fastq_bytes(synth.workload("plain_small", 2000, seed=7))
    i = torch.frombuffer(bytearray(data), dtype=torch.uint8).pin_memory()
    o = torch.empty(len(data) + 64, dtype=torch.uint8).pin_memory()
    with serve.Server(ctx, slots=1) as srv:
        t = srv.submit(i.data_ptr(), i.numel(), serve.RequestParams(27, 0, 1, 1, 2, 0), o.data_ptr(), o.numel())
        assert srv.result(t).status == 0
        for wait in (False, True):
            with pytest.raises(native.MetapartError):
                srv.result(t, wait=wait)
        with pytest.raises(native.MetapartError):
            srv.result(t + 1000, wait=True)


def native_code(name):
    return {"MP_EARG": -1, "MP_ENOMEM": -4}[name]
