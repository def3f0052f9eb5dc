"""One rank of bench.py's N-replica timing on the CPU (gloo), launched by torchrun from
tests/test_replicas.py: rank r contributes a timed region of 1.5 + r seconds over 30 frames and
writes what bench.py's helpers make of it (the slowest rank's time, the whole-job rate) to
rank<r>.json in the directory given as the argument (the ranks share one stdout)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

world = int(os.environ["WORLD_SIZE"])
rank = int(os.environ["RANK"])
dist = bench.dist_setup(world, backend="gloo")
assert dist is not None and dist.get_world_size() == world
slowest = bench.max_over_ranks(1.5 + rank, dist, "cpu")
with open(os.path.join(sys.argv[1], "rank%d.json" % rank), "w") as fh:
    json.dump({"rank": rank, "world": world, "max_seconds": slowest,
               "frames_per_s": bench.whole_job_rate(30, world, slowest)}, fh)
dist.destroy_process_group()
