"""Host logic of the pipelined learned stream (no GPU): the order of the
stages of consecutive batches, the alternation of contexts and outputs, and
the clean-up when a stage fails or the caller stops early.  The batch stages
are replaced by a recorder; the GPU form is tested in test_learned.py."""
import pytest

from grtm_cuda_gb300 import learned


class _Rec:
    log = []
    fail_finish = None

    def __init__(self, sampler, models, dists_list, ctx, plain, spec_tol, autotune, use_stride, out):
        self.name, self.ctx, self.out = models, ctx, out
        _Rec.log.append(("make", models))

    def start(self, threaded=True):
        _Rec.log.append(("start", self.name))

    def judge_pre(self, jctx):
        assert jctx == "judge"
        _Rec.log.append(("judge", self.name))

    def wait_stages(self):
        _Rec.log.append(("stages", self.name))

    def join(self):
        _Rec.log.append(("join", self.name))

    def finish(self, overlap):
        assert overlap
        _Rec.log.append(("finish", self.name))
        if _Rec.fail_finish == self.name:
            raise RuntimeError("finish failed")
        return [self.name], {"ctx": self.ctx, "out": self.out}

    def abandon(self):
        _Rec.log.append(("abandon", self.name))


@pytest.fixture
def rec(monkeypatch):
    _Rec.log, _Rec.fail_finish = [], None
    monkeypatch.setattr(learned, "_LearnedBatch", _Rec)
    monkeypatch.setattr(learned, "judge_context", lambda ctx: "judge")
    return _Rec


def _work(n):
    return [(i, None) for i in range(n)]


def test_stream_order_and_alternation(rec):
    got = []
    for traces, info in learned.run_learned_stream(None, _work(3), ("c0", "c1"), outs=("o0", "o1")):
        got.append((traces[0], info["ctx"], info["out"]))
        rec.log.append(("yield", traces[0]))
    assert got == [(0, "c0", "o0"), (1, "c1", "o1"), (2, "c0", "o0")]
    # batch i+1 is built and judged before batch i's stages end, its graph
    # starts before batch i's comparison, and results come out in order
    assert rec.log == [
        ("make", 0), ("start", 0), ("judge", 0),
        ("make", 1), ("judge", 1), ("stages", 0), ("start", 1), ("join", 0), ("finish", 0), ("yield", 0),
        ("make", 2), ("judge", 2), ("stages", 1), ("start", 2), ("join", 1), ("finish", 1), ("yield", 1),
        ("stages", 2), ("join", 2), ("finish", 2), ("yield", 2)]


def test_stream_failure_abandons_running_batches(rec):
    rec.fail_finish = 1
    it = learned.run_learned_stream(None, _work(4), ("c0", "c1"))
    assert next(it)[0] == [0]
    with pytest.raises(RuntimeError, match="finish failed"):
        next(it)
    # batch 1 failed in its comparison while batch 2's graph ran: both are
    # waited for and freed, nothing after them is built
    assert rec.log[-3:] == [("finish", 1), ("abandon", 1), ("abandon", 2)]
    assert ("make", 3) not in rec.log


def test_stream_early_stop_abandons_the_running_batch(rec):
    it = learned.run_learned_stream(None, _work(3), ("c0", "c1"))
    assert next(it)[0] == [0]
    it.close()                               # the caller stops after one batch
    assert rec.log[-1] == ("abandon", 1)
    assert ("make", 2) not in rec.log


def test_stream_edge_cases(rec):
    assert list(learned.run_learned_stream(None, [], ("c0", "c1"))) == []
    with pytest.raises(ValueError):
        list(learned.run_learned_stream(None, _work(1), ("c0",)))
    assert [t for t, _ in learned.run_learned_stream(None, _work(1), ("c0", "c1"))] == [[0]]
