"""The sweep autotuner's host logic (BatchTuner): it times each candidate lane
count on a real interval, keeps the fastest, caches it per device and size
profile, and reuses the cache without timing.  A stand-in batch whose interval
time depends on the lane count replaces the CUDA batch, so no GPU is needed."""

import json
import time
from types import SimpleNamespace

import pytest

from blademaster_gb300.batch import BatchTuner


class FakeBatch:
    """Intervals take longer the further the lane count is from `best`."""

    def __init__(self, sizes, best):
        self.solvers = [SimpleNamespace(n=n, config=SimpleNamespace(dt=6.25e-5)) for n in sizes]
        self.device = "cuda:0"
        self.best = best
        self.lanes = None
        self.graphs, self.advanced = [], []

    def graph(self, steps, cutting, cut_index, lanes):
        self.graphs.append((tuple(steps), lanes))

    def advance(self, states, duration_s, lanes=None, **kw):
        time.sleep(0.002 + 0.02 * abs(lanes.bit_length() - self.best.bit_length()))
        self.advanced.append(lanes)
        return [f"reaction {i}" for i in range(len(states))]


@pytest.fixture
def no_cuda(monkeypatch):
    import torch

    monkeypatch.setattr(torch.cuda, "get_device_name", lambda device=None: "GB300 stand-in")
    monkeypatch.setattr(torch.cuda, "synchronize", lambda device=None: None)


def states_for(i):
    return [i] * 3


def test_tuner_keeps_the_fastest_candidate_and_caches_it(tmp_path, no_cuda):
    cache = tmp_path / "tune.json"
    batch = FakeBatch([4480, 11024, 35840] * 12, best=32)  # 36 instances: 64 and 128 lanes are skipped
    tuner = BatchTuner(cache=cache)
    reactions = tuner.tune(batch, states_for, 0.001, strict=False)
    assert batch.advanced == [8, 16, 32]
    assert batch.lanes == 32
    assert len(reactions) == 3 and reactions[0][0] == "reaction 0"
    assert all(steps == (16,) * 36 for steps, _ in batch.graphs)
    table = json.loads(cache.read_text())
    assert list(table.values()) == [32]
    assert set(tuner.timings) == {8, 16, 32}

    again = FakeBatch([4480, 11024, 35840] * 12, best=8)
    assert BatchTuner(cache=cache).tune(again, states_for, 0.001) == []
    assert again.lanes == 32 and again.advanced == []  # the cached choice, no timing


def test_signature_separates_size_profiles(no_cuda):
    a = BatchTuner.signature(FakeBatch([4480] * 16, best=8))
    b = BatchTuner.signature(FakeBatch([4480] * 8 + [35840] * 8, best=8))
    c = BatchTuner.signature(FakeBatch([4480] * 32, best=8))
    assert len({a, b, c}) == 3


def test_corrupt_cache_is_ignored(tmp_path, no_cuda):
    cache = tmp_path / "tune.json"
    cache.write_text("{not json")
    batch = FakeBatch([4480] * 20, best=16)
    BatchTuner(cache=cache, candidates=(8, 16)).tune(batch, states_for, 0.001)
    assert batch.lanes == 16
    assert list(json.loads(cache.read_text()).values()) == [16]
