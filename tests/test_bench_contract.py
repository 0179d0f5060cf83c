"""The benchmark's reference arm on CPU: one JSON line with the keys the
benchmark contract asks for (metric, unit, timing, config, cpu_baseline,
e2e with zero copies), and the other ranks of a multi-rank launch print
nothing."""
import json
import os
import subprocess
import sys

from conftest import REPO


def _run(env_extra=None, *args):
    env = dict(os.environ)
    env.update(env_extra or {})
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", *args], capture_output=True, text=True, env=env, timeout=600, check=True)
    return [l for l in out.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line():
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["higher_is_better"] is True and d["vs_baseline"] is None
    # the reference's own stage bodies when their host build is present
    # (staged reference sources), else the oracle restatement
    import oracle as O
    want = "reference" if (O.ref_available(5) and O.ref_available(48)) else "port"
    assert d["cpu_baseline"]["kind"] == want and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]


def test_reference_arm_other_ranks_are_silent():
    assert _run({"RANK": "1", "WORLD_SIZE": "2"}) == []
