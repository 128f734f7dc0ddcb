"""The autotuner's search and choice (govid_gb300/autotune.py) on CPU, with
the measurement replaced by a table: it tries lookahead x depth first, then
entropy launches x intra warps at the best of those, and picks by its
objective."""
from govid_gb300 import autotune


def fake_trials(table):
    calls = []

    def trial(streams, lookahead, depth, groups, warps, frames):
        calls.append((lookahead, depth, groups, warps))
        fps, p99 = table(lookahead, depth, groups, warps)
        return {"lookahead": lookahead, "pipeline_depth": depth, "entropy_groups": groups, "intra_warps": warps,
                "frames_per_s": fps, "round_p99_ms": p99, "round_p50_ms": p99 / 2}

    return trial, calls


def test_throughput_objective_takes_the_fastest_setting(monkeypatch):
    # fastest at lookahead 4, depth 2, then 2 entropy launches and 16 warps
    def table(la, d, g, w):
        fps = 1000 * la * (1.5 if d == 2 else 1.0) / (1 + (la == 8))
        if (g, w) == (2, 16):
            fps *= 1.2
        return fps, 5.0 * la

    trial, calls = fake_trials(table)
    monkeypatch.setattr(autotune, "_trial", trial)
    r = autotune.tune([[b"x"]], frames=4)
    assert r["choice"]["lookahead"] == 4 and r["choice"]["pipeline_depth"] == 2
    assert (r["choice"]["entropy_groups"], r["choice"]["intra_warps"]) == (2, 16)
    first = [(la, d) for la, d, g, w in calls[: len(autotune.LOOKAHEADS) * len(autotune.DEPTHS)]]
    assert sorted(first) == sorted((la, d) for la in autotune.LOOKAHEADS for d in autotune.DEPTHS)
    assert all((la, d) == (4, 2) for la, d, g, w in calls[len(first):])  # second stage at the best shape
    assert len(r["trials"]) == len(calls)


def test_latency_objective_respects_the_round_budget(monkeypatch):
    # faster settings have longer rounds; the budget keeps lookahead <= 2
    def table(la, d, g, w):
        return 1000.0 * la, 8.0 * la

    trial, _ = fake_trials(table)
    monkeypatch.setattr(autotune, "_trial", trial)
    r = autotune.tune([[b"x"]], objective="latency", round_budget_ms=16.7)
    assert r["choice"]["lookahead"] == 2 and r["choice"]["round_p99_ms"] <= 16.7
    # nothing within budget: the fastest setting
    r = autotune.tune([[b"x"]], objective="latency", round_budget_ms=1.0)
    assert r["choice"]["lookahead"] == max(autotune.LOOKAHEADS)
