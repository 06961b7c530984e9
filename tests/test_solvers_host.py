"""Host-side logic of the solvers module that needs no GPU: the job queue of
solve_batches (largest job first, results in job order, errors raised on the caller's
thread), with the per-operator batched solve and the CUDA stream objects replaced by
fakes."""
import contextlib
import threading

import pytest


class _Stream:
    def wait_stream(self, other):
        pass

    def synchronize(self):
        pass


class _Op:
    def __init__(self, name, segments):
        self.name = name
        self.ICn = segments
        self.ICnRF = 1
        self.device = 0


@pytest.fixture
def fake_cuda(monkeypatch):
    from commit_gb300 import solvers
    monkeypatch.setattr(solvers.torch.cuda, 'Stream', lambda device=None: _Stream())
    monkeypatch.setattr(solvers.torch.cuda, 'current_stream', lambda device=None: _Stream())
    monkeypatch.setattr(solvers.torch.cuda, 'device', lambda d: contextlib.nullcontext())
    monkeypatch.setattr(solvers.torch.cuda, 'stream', lambda s: contextlib.nullcontext())
    return solvers


def _jobs():
    # work = segments x problems: a 20, b 100, c 150, d 40
    return [(None, _Op('a', 10), [1, 2]), (None, _Op('b', 100), [1]), (None, _Op('c', 50), [1, 2, 3]),
            (None, _Op('d', 40), [7])]


def test_solve_batches_order_and_results(fake_cuda, monkeypatch):
    solvers = fake_cuda
    started, lock = [], threading.Lock()

    def fake_solve_batch(y, A, regs, **kw):
        with lock:
            started.append(A.name)
        return [(A.name, r, kw.get('max_iter')) for r in regs]

    monkeypatch.setattr(solvers, 'solve_batch', fake_solve_batch)
    out = solvers.solve_batches(_jobs(), n_streams=1, max_iter=5)
    assert started == ['c', 'b', 'd', 'a']  # largest first
    assert out == [[('a', 1, 5), ('a', 2, 5)], [('b', 1, 5)], [('c', 1, 5), ('c', 2, 5), ('c', 3, 5)],
                   [('d', 7, 5)]]
    started.clear()
    out4 = solvers.solve_batches(_jobs(), n_streams=4, max_iter=5)
    assert out4 == out and sorted(started) == ['a', 'b', 'c', 'd']
    assert solvers.solve_batches([], n_streams=4) == []


def test_solve_batches_raises_a_job_error(fake_cuda, monkeypatch):
    solvers = fake_cuda

    def failing(y, A, regs, **kw):
        if A.name == 'b':
            raise RuntimeError('job b failed')
        return [None] * len(regs)

    monkeypatch.setattr(solvers, 'solve_batch', failing)
    for n in (1, 3):
        with pytest.raises(RuntimeError, match='job b failed'):
            solvers.solve_batches(_jobs(), n_streams=n)
