"""bench.py --gpus N started without torchrun launches N local ranks itself
(torch.distributed.run, 127.0.0.1).  With --plan-only every rank builds its
slice of the workload and rank 0 prints the gathered slices; on CPU the ranks
use gloo.  The ensemble is split by systems: rank r owns disks
[512 r, 512 (r + 1)), so the ranks' first disks differ."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(600)
def test_bench_starts_n_ranks():
    pytest.importorskip("torch")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    env.pop("WORLD_SIZE", None)
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--config", "c4",
                        "--plan-only"], capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    ranks = sorted(d["ranks"], key=lambda r: r["rank"])
    assert [r["rank"] for r in ranks] == [0, 1] and all(r["world"] == 2 for r in ranks)
    assert all(r["systems"] == 512 for r in ranks)
    assert ranks[0]["first_x"] != ranks[1]["first_x"]
