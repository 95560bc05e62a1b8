"""The benchmark's host-side pieces that need no GPU: the figures it reads
from the committed profile summaries (the FP64 operator count the CPU
baseline is projected onto, the ncu DRAM traffic of one operator launch),
the reduction of a timing over ranks with world_size-1, and the shape of
the reference arm's output when that count is missing."""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_profile_notes_carry_the_recorded_figures():
    n = bench._recorded_fp64_matvecs()
    assert isinstance(n, int) and n > 1000
    t = bench._recorded_traffic()
    assert isinstance(t, float) and t > 0
    # the traffic of one launch is below the algorithmic bytes of the 96³
    # workload (60 B/cell + 12 B per flagged corner, ≥ 53 MB): no re-reads
    assert t < 60 * 96 ** 3


def test_reference_arm_without_recorded_count(monkeypatch, capsys):
    monkeypatch.setattr(bench, "_recorded_fp64_matvecs", lambda: None)
    monkeypatch.setattr(bench, "_dist", lambda: (1, 0, 0))

    class Args:
        gpus, steps, warmup = 1, 1, 0

    assert bench.run_reference(Args()) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line


def test_cpu_model_is_named():
    assert isinstance(bench._cpu_model(), str) and bench._cpu_model()


@pytest.mark.parametrize("value", [0.5, 3.25])
def test_max_over_ranks_single_process(value):
    assert bench.max_over_ranks(value, 1) == value
