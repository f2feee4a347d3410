"""Host logic of the recording integration's record growth (BatchIntegrator.record) with a CPU stand-in for the
device launch: reactors that fill their record are integrated again by themselves into a larger record, and the
merged results equal those of one launch whose record fits every reactor."""
import numpy as np
import torch

from spitfire_gb300.reactors import BatchIntegrator

NEQ = 3


class FakeIntegrator:
    """allocate/launch with the device calls' contract: reactor i takes steps(q0[i]) accepted steps and writes
    row k of its record as (t_k, h_k, stage values); a reactor whose steps exceed the capacity stops at the
    capacity with status 7 (its results are then those of a partial run)."""

    def __init__(self):
        self.launched = []

    @staticmethod
    def steps(q):
        return int(q[0]) % 37 + 5

    def allocate(self, n):
        return dict(q=torch.empty((n, NEQ), dtype=torch.float64), t=torch.empty(n, dtype=torch.float64),
                    t_interp=torch.full((n,), float('nan'), dtype=torch.float64),
                    counts=torch.empty((n, 4), dtype=torch.int32), status=torch.empty(n, dtype=torch.int32),
                    ws=torch.empty(1, dtype=torch.int32))

    def launch(self, q0, pressures, out, ip, record=None):
        cap = record.shape[1]
        self.launched.append((q0.shape[0], cap))
        for i in range(q0.shape[0]):
            k = self.steps(q0[i])
            done = min(k, cap)
            for s in range(done):
                record[i, s, 0] = 0.5 * s
                record[i, s, 1] = 0.5
                record[i, s, 2:] = float(q0[i, 0]) + s + (0. if pressures is None else float(pressures[i]))
            out['q'][i] = q0[i] + done
            out['t'][i] = 0.5 * done
            out['t_interp'][i] = 0.25 * done
            out['counts'][i] = torch.tensor([done, 2 * done, done, 0], dtype=torch.int32)
            out['status'][i] = 7 if k > cap else 1


def test_growth_reruns_only_full_reactors_and_matches_one_fitting_run():
    rng = np.random.default_rng(3)
    n = 40
    q0 = torch.from_numpy(np.hstack([rng.integers(0, 1000, (n, 1)).astype(float), rng.random((n, NEQ - 1))]))
    p = torch.from_numpy(rng.random(n))
    f = FakeIntegrator()
    out, rec = BatchIntegrator.record(f, q0, p, None, 8)
    steps = np.array([FakeIntegrator.steps(q) for q in q0])
    assert rec.shape[1] >= steps.max()
    # the first launch covers the batch, each later one only the reactors still out of room
    assert f.launched[0] == (n, 8)
    for (m0, c0), (m1, c1) in zip(f.launched, f.launched[1:]):
        assert m1 <= m0 and c1 == 2 * c0
    assert f.launched[1][0] == int((steps > 8).sum())
    ref = FakeIntegrator()
    rout, rrec = BatchIntegrator.record(ref, q0, p, None, 64)
    assert ref.launched == [(n, 64)]
    for k in ('q', 't', 't_interp', 'counts', 'status'):
        assert torch.equal(out[k], rout[k]), k
    for i in range(n):
        assert torch.equal(rec[i, :steps[i]], rrec[i, :steps[i]])
    assert (out['status'] == 1).all()


def test_growth_without_pressures_and_for_an_empty_batch():
    f = FakeIntegrator()
    q0 = torch.tensor([[40., 0.1, 0.2], [3., 0.3, 0.4]], dtype=torch.float64)
    out, rec = BatchIntegrator.record(f, q0, None, None, 4)
    assert out['counts'][:, 0].tolist() == [FakeIntegrator.steps(q) for q in q0]
    e = FakeIntegrator()
    out, rec = BatchIntegrator.record(e, torch.empty((0, NEQ), dtype=torch.float64), None, None, 16)
    assert rec.shape == (0, 16, 2 + 6 * NEQ) and e.launched == [(0, 16)]


def test_starting_capacity_fits_a_share_of_free_memory():
    from spitfire_gb300.reactors import record_capacity
    row = (2 + 6 * 53) * 8
    assert record_capacity(2048, 53, 270e9) == 1024                    # 5.4 GB of a 67.5 GB share
    assert record_capacity(100000, 53, 270e9) == 256                   # 100 k reactors: 65.5 GB at 256 steps
    assert 100000 * 256 * row <= 0.25 * 270e9 < 100000 * 512 * row
    assert record_capacity(10 ** 7, 53, 1e9) == 64                     # never below 64 steps
    assert record_capacity(1, 53, 270e9, most=4096) == 4096
