"""The benchmark's host-side pieces that need no GPU: the reference (CPU)
arm's output line — a measured complete solve, not a projection — on a small
stand-in system, the reduction of a timing over ranks with world_size-1, and
that the script reads no figure out of the profile summaries."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_times_a_complete_solve(monkeypatch, capsys, oracle):
    from oracle.build_oracle import build
    from oracle.csr_native import NativeCSR
    build()
    O = oracle
    g = O.uniform_grid((14, 12, 10))
    S = O.System(g, 2 * np.pi / 8, ((3, 3, 3), (3, 3, 3)), [O.Sphere((7.1, 6.2, 5.3), 3.0, 6.0)])
    S.add_planesrc(2, 4.0, (1, 0, 0))
    monkeypatch.setattr(bench, "_CPU", {"b": S.b(), "M": NativeCSR(S.A, threads=2), "t_asm": 0.0})
    monkeypatch.setattr(bench, "_dist", lambda: (1, 0, 0))

    class Args:
        gpus, steps, warmup = 1, 2, 1

    assert bench.run_reference(Args()) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["cpu_relres"] <= 1e-6 and line["cpu_matvecs"] > 0
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert "complete" in line["cpu_baseline"]["sample"]


def test_bench_reads_no_profile_summary():
    with open(os.path.join(ROOT, "bench.py")) as f:
        src = f.read()
    assert "profiles/" not in src.replace("kept in profiles/", "")


def test_cpu_model_is_named():
    assert isinstance(bench._cpu_model(), str) and bench._cpu_model()


@pytest.mark.parametrize("value", [0.5, 3.25])
def test_max_over_ranks_single_process(value):
    assert bench.max_over_ranks(value, 1) == value
