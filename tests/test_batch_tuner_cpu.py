"""Bookkeeping of the batched solve's worker-count autotuner (no GPU: the
batch call is replaced by a stand-in whose time depends on the count)."""
import time

import pytest

from bem_gmsh_gb300 import api
from bem_gmsh_gb300.geometry import c4_domains, c4_node_counts


@pytest.fixture
def fake_batch(monkeypatch):
    calls = []

    def fake(dads, npg=20, mode="mixed", nworkers=0, ctx=None, **kw):
        calls.append(nworkers)
        time.sleep({2: 0.03, 4: 0.005, 8: 0.02}.get(nworkers, 0.04))
        return []
    monkeypatch.setattr(api, "solve_batch", fake)
    monkeypatch.setattr(api, "_BATCH_TUNED", {})
    return calls


def test_tuner_picks_fastest_and_caches_per_shape(fake_batch):
    dads = c4_domains(c4_node_counts(6, hi=300, seed=1))
    best, times = api.tune_batch(dads, npg=16, candidates=(8, 2, 4, 99), repeats=2)
    assert best == 4
    assert sorted(times) == [2, 4, 8]           # 99 is outside 1..32 and dropped
    assert fake_batch[0] == 8                   # warm-up at the largest count
    assert fake_batch[1:] == [2, 2, 4, 4, 8, 8]
    assert api.batch_workers(dads, 16, "mixed") == 4
    # another rule, mode or batch size class falls back to the default
    assert api.batch_workers(dads, 20, "mixed") == api.BATCH_WORKERS_DEFAULT
    assert api.batch_workers(dads, 16, "fp64") == api.BATCH_WORKERS_DEFAULT
    big = c4_domains(c4_node_counts(40, hi=300, seed=1))
    assert api.batch_workers(big, 16, "mixed") == api.BATCH_WORKERS_DEFAULT


def test_tuner_rejects_empty_input(fake_batch):
    with pytest.raises(ValueError):
        api.tune_batch([], candidates=(2,))
    dads = c4_domains(c4_node_counts(3, hi=200, seed=2))
    with pytest.raises(ValueError):
        api.tune_batch(dads, candidates=(0, 64))


def test_adjoint_batch_argument_checks_run_on_the_host():
    # rejected before any library call (no GPU needed)
    import numpy as np
    from bem_gmsh_gb300 import star_adjoint_case
    from bem_gmsh_gb300.geometry import quadrado
    d, _ = star_adjoint_case(20, p=2, seed=1)
    assert api.adjoint_laplace_batch([]) == []
    assert api.adjoint_laplace_batch([], return_stats=True) == ([], [])
    with pytest.raises(ValueError):
        api.adjoint_laplace_batch([(d, np.zeros(d.n + 1))])
    with pytest.raises(ValueError):          # internal points are not supported
        q = quadrado(ndiv=5)
        api.adjoint_laplace_batch([(q, np.zeros(q.n))])
