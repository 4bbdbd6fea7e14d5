"""The N-rank path of bench.py on CPU ranks (gloo, world size 2): the path
does not shard inside a step, so N ranks run independent replicas (one kick
direction each) joined only by a barrier and the max / sum over ranks of the
timing and the work done."""
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK = textwrap.dedent(r"""
    import os, sys
    sys.path.insert(0, os.environ["OPAW_ROOT"])
    import bench
    rank, world, local = bench.dist_env()
    dist = bench.init_dist(world)
    assert dist is not None and dist.get_world_size() == 2
    bench.barrier(dist)
    mx = bench.max_over_ranks(dist, 1.5 + rank)          # the slowest rank's time
    sm = bench.sum_over_ranks(dist, 2.0 * 128 * (rank + 1))  # work of all replicas
    assert mx == 2.5, mx
    assert sm == 2.0 * 128 * 3, sm
    ipol = 1 + (rank % 3)  # replicas kick along x, y, z in turn
    import torch
    t = torch.zeros(2, dtype=torch.float64)
    t[rank] = ipol
    dist.all_reduce(t)
    assert t.tolist() == [1.0, 2.0], t
    # the reference arm under N ranks: rank 0 alone runs and prints
    if rank == 1:
        class A:
            steps, warmup, gpus = 1, 1, 2
        assert bench.run_reference(A()) == 0
    bench.barrier(dist)
    dist.destroy_process_group()
    print("rank", rank, "ok")
""")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replica_ranks_gloo(tmp_path):
    script = tmp_path / "rank.py"
    script.write_text(_RANK)
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), OPAW_ROOT=ROOT, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = []
    for p in procs:
        try:
            out, _ = p.communicate(timeout=240)
        except subprocess.TimeoutExpired:
            p.kill()
            out, _ = p.communicate()
        outs.append(out)
    for r, (p, out) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, out
        assert f"rank {r} ok" in out, out
    # rank 1 of the reference arm printed nothing
    assert '"impl": "reference"' not in outs[1]
