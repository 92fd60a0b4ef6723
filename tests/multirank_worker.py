"""Worker of tests/test_multirank.py: one gloo rank of a CPU process group."""
import os
import sys


def run(rank: int, world: int, port: int, out_dir: str) -> None:
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        # each rank reports a different step time; every rank must see the slowest
        slowest = bench.max_over_ranks(1.5 + rank, "cpu")
        rate = bench.replicas_rate(world, 1000.0, slowest)
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as fp:
            fp.write(f"{slowest} {rate}\n")
    finally:
        dist.destroy_process_group()
