"""The bounded device waits run out and report it, and the context stays usable.

Every device wait has an iteration limit (mp_job_set_wait_limits): the sort's decoupled look-back polls of
a predecessor tile's status word, the union-find's hook attempts of one union, the mate union's rounds.
Here each limit is set to 1 on an input where the wait is certain to be needed more than once -- tens of
millions of tuples for the look-back (a tile finding its predecessor's count not yet posted), runs of
equal k-mers from one 200 bp genome at very high coverage for the unions (lanes hooking the same root at
once), thousands of pairs for the mate union -- and the partition must return MP_EDEVICE with a message
naming the wait.  Nothing spins without a limit: a look-back that gives up still posts its tile's prefix
for its successors, a union that gives up returns, the mate-union loop stops on the host.  After each
failure a fresh run on the same context (the job reset, default limits) must give the results of a run
that never failed.
"""
import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu

CASES = [
    # limit, workload, reads, k, message
    ("lookback", "plain_large", 200_000, 31, "look-back"),
    ("union", "hotspot", 40_000, 27, "union-find"),
    ("mate", "plain_small", 20_000, 27, "mate union"),
]


def _partition(ctx, data, k, limits=None):
    fno, ofs = native.fastq_index(8, [data])
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as job:
        if limits:
            job.set_wait_limits(**limits)
        job.load(data)
        cnt = job.count(k, starts)
        bounds = job.partition(k, 1, 4, starts, cnt.chunk_first_read, cnt.hist)
        return bounds, job.labels()


@pytest.mark.parametrize("which,work,n,k,msg", CASES, ids=[c[0] for c in CASES])
def test_bounded_wait_runs_out_and_context_recovers(built_gpu, which, work, n, k, msg):
    data = synth.fastq_bytes(synth.workload(work, n, seed=31))
    lim = {"lookback": {"lookback_spins": 1}, "union": {"union_retries": 1}, "mate": {"mate_rounds": 1}}[which]
    with native.Context(0) as ctx:
        want_b, want_l = _partition(ctx, data, k)
        with pytest.raises(native.MetapartError, match=msg) as ei:
            _partition(ctx, data, k, lim)
        assert "(-7)" in str(ei.value)  # MP_EDEVICE
        got_b, got_l = _partition(ctx, data, k)
        assert np.array_equal(got_b, want_b) and np.array_equal(got_l, want_l)
