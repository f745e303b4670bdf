"""Host logic of the autotuner (no GPU): candidate enumeration, child
failures, choice of the fastest candidate."""
import json
import subprocess

from stan_gb300 import autotune


def test_sweep_picks_fastest_and_reports_failures(monkeypatch):
    calls = []

    class R:
        def __init__(self, rc, out, err=""):
            self.returncode, self.stdout, self.stderr = rc, out, err

    def fake_run(cmd, cwd, capture_output, text, timeout):
        sr = int(cmd[cmd.index("--split-rows") + 1])
        tw = int(cmd[cmd.index("--team-warps") + 1])
        calls.append((sr, tw))
        assert "--child" in cmd
        if sr == 128 and tw == 4:
            return R(1, "", "boom")
        ms = abs(sr - 256) / 100 + tw * 0.1
        return R(0, "noise\n" + json.dumps({"ms_per_step": ms, "grad_ms": 0.1, "steps": 10}))

    monkeypatch.setattr(subprocess, "run", fake_run)
    rows, best = autotune.sweep("hier_normal", 256, "fp32", split_rows=(128, 256),
                                team_warps=(1, 4))
    assert calls == [(128, 1), (128, 4), (256, 1), (256, 4)]
    assert best["split_rows"] == 256 and best["team_warps"] == 1
    assert "error" in rows[1] and "boom" in rows[1]["error"]
