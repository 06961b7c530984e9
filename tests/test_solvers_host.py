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


def test_solve_mixed_joins_the_phases(monkeypatch):
    """solve_mixed: phase 2 starts from phase 1's x with the refinement settings, the
    iterations add up, and with x_ref the two traces (seconds, |x - x_ref| / |x_ref|, cost)
    join into one, phase 2's times shifted by phase 1's duration."""
    import numpy as np
    from commit_gb300 import solvers
    calls = []

    def fake_solve(y, A, At, tol_fun, tol_x, max_iter, verbose, x0, regularisation, confidence_array, arith, x_ref,
                   restart):
        calls.append(dict(x0=x0, arith=arith, max_iter=max_iter, tol_fun=tol_fun, restart=restart))
        n = 3 if len(calls) == 1 else 2
        tr = np.array([[0.1 * (k + 1), 1.0 / (k + 2), 10.0 - k] for k in range(n)])
        return np.full(4, float(len(calls))), {'iterations': n, 'trace': tr, 'cost_function': 1.0}

    monkeypatch.setattr(solvers, 'solve', fake_solve)

    class _A:
        T = None

    x, det = solvers.solve_mixed(None, _A(), tol_fun=1e-4, max_iter=7, arith='bf16', refine_max_iter=5,
                                 refine_tol_fun=1e-6, x_ref=np.ones(4), restart=True)
    assert calls[0]['arith'] == 'bf16' and calls[0]['x0'] is None and calls[0]['max_iter'] == 7
    assert calls[1]['arith'] is None and np.array_equal(calls[1]['x0'], np.full(4, 1.0))
    assert calls[1]['max_iter'] == 5 and calls[1]['tol_fun'] == 1e-6 and calls[1]['restart']
    assert det['iterations'] == 5 and np.array_equal(x, np.full(4, 2.0))
    tr = det['trace']
    assert tr.shape == (5, 3)
    shift = tr[3:, 0] - det['refine']['trace'][:, 0]  # phase 1's duration, added to phase 2's times
    assert shift[0] > 0 and np.allclose(shift, shift[0])
    assert np.array_equal(tr[:3], det['mixed']['trace'])
    assert np.allclose(tr[3:, 1:], det['refine']['trace'][:, 1:])
