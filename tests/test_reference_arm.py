"""The bench's reference arm: the oracle's onestep (the reference's
algorithm on the host cores) timed with the bench's warm-up and step
counts, on a small slab so that it runs in a fraction of a second here."""
from __future__ import annotations

import math
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_run_honours_warmup_and_steps(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    calls = []
    real = bench._oracle_sample

    def counted(o, t_nl, first, sample_steps, nthreads, state):
        calls.append((first, sample_steps))
        return real(o, t_nl, first, sample_steps, nthreads, state)

    monkeypatch.setattr(bench, "_oracle_sample", counted)
    value, cb = bench.cpu_reference_run((4, 4, 4), 2, 3, 2, nthreads=2)
    # two untimed and three timed samples of two steps each, consecutive
    assert calls == [(0, 2), (2, 2), (4, 2), (6, 2), (8, 2)]
    assert math.isfinite(value) and value > 0
    assert cb["value"] == value and cb["cores"] == 2 and cb["kind"] == "port"
    assert "median of 3 steps after 2 untimed" in cb["sample"]


def test_cpu_baseline_after_an_untimed_sample(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    calls = []
    real = bench._oracle_sample

    def counted(o, t_nl, first, sample_steps, nthreads, state):
        calls.append(first)
        return real(o, t_nl, first, sample_steps, nthreads, state)

    monkeypatch.setattr(bench, "_oracle_sample", counted)
    cb = bench.cpu_baseline((4, 4, 4), 3, nthreads=2)
    assert calls == [0, 3]
    assert cb["value"] > 0 and cb["unit"] == "atom-steps/s"
