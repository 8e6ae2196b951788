"""Batched replicas (hymd_gb300.replicas): one captured graph advancing all
replicas concurrently gives bit-identical trajectories to the same replicas
stepped one by one (every kernel on the path is deterministic)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _systems():
    from hymd_gb300 import systems
    return systems.replica_set(n_replicas=6, seed=11, n_min=2000, n_max=40000)


def test_batched_replicas_match_replica_by_replica():
    from hymd_gb300.replicas import ReplicaBatch
    a = ReplicaBatch(_systems(), seed=3)
    b = ReplicaBatch(_systems(), seed=3)
    assert len({md.pm.Nmesh for md in a.replicas}) >= 2  # mixed mesh sizes
    for x in (a, b):
        x.prime()
    a.capture(n_streams=4)
    b.capture_each()
    a.run(3)
    b.run_sequential(3)
    torch.cuda.synchronize()
    for ra, rb in zip(a.replicas, b.replicas):
        assert torch.equal(ra.r, rb.r)
        assert torch.equal(ra.v, rb.v)
        assert np.isfinite(ra.r.cpu().numpy()).all()
    a.check_errors()
    b.check_errors()


def test_stream_tuning_picks_a_measured_candidate():
    from hymd_gb300.replicas import ReplicaBatch
    a = ReplicaBatch(_systems(), seed=4)
    a.prime()
    k = a.tune_streams(candidates=(2, 3, 6), reps=1)
    assert k in a.stream_timings and a.stream_timings[k] == min(a.stream_timings.values())
    assert len(a.step_us) == 6 and all(t > 0 for t in a.step_us)
    a.run(2)
    torch.cuda.synchronize()
    a.check_errors()
