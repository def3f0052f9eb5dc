"""bench.py's N-replica path on the CPU, launched the way an N-GPU run is (torchrun, one process per
rank, rendezvous on 127.0.0.1), with the gloo backend and world size 2: the timed region is the
slowest rank's on every rank, `value` is the whole job's rate (weak scaling: every replica fuses the
same sequence), and the reference arm runs and prints on rank 0 alone, on every host thread, while
the other ranks exit 0 without work.  The path does not shard inside a session, so there is no
data-path collective to test: replicas only."""
import json
import os
import socket
import subprocess
import sys

import pytest

pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, PYTHONUNBUFFERED="1")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def _json_lines(text):
    out = []
    for line in text.splitlines():
        line = line.strip()
        if line.startswith("{"):
            out.append(json.loads(line))
    return out


def test_slowest_rank_and_whole_job_rate_gloo(tmp_path):
    p = _torchrun([os.path.join("tests", "_replica_worker.py"), str(tmp_path)])
    assert p.returncode == 0, p.stdout + p.stderr
    lines = [json.loads((tmp_path / ("rank%d.json" % r)).read_text()) for r in range(2)]
    assert [d["rank"] for d in lines] == [0, 1]
    for d in lines:
        assert d["world"] == 2
        assert d["max_seconds"] == 2.5  # rank 1's 2.5 s, seen by both ranks
        assert d["frames_per_s"] == 2 * 30 / 2.5


def test_reference_arm_prints_once_from_rank_zero():
    p = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--clip", "2"])
    assert p.returncode == 0, p.stdout + p.stderr
    lines = _json_lines(p.stdout)
    assert len(lines) == 1, p.stdout
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    # torchrun sets OMP_NUM_THREADS=1 for its processes; the reference arm still uses every host thread
    assert d["cpu_baseline"]["cores"] == os.cpu_count()
