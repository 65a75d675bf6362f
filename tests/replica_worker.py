"""One rank of the replicas test: run by test_replicas_gloo.py as two processes with RANK,
WORLD_SIZE, LOCAL_RANK and MASTER_ADDR/PORT set, over the gloo backend on the CPU.  Drives
bench.py's multi-process helpers (process group, barriers, max-over-ranks timing, per-rank
frames, the reference arm that rank 0 alone runs) and writes what it saw to <out>/rank<r>.json.

    python tests/replica_worker.py <out-dir>
"""
import contextlib
import hashlib
import io
import json
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402

# a frame small enough for the oracle to finish in well under a second
TINY = dict(name="plain-64x48-rggb12-5lvl", width=64, height=48, bayer=2, bits=12, black=64, white=4095,
            wb=(2.0, 1.0, 1.6), noise=[(2.0, 1.0, 0.2), (6.0, 4.0, 0.45), (12.0, 16.0, 0.7)], levels=5,
            storage=0, out="rgba8")


def main(out_dir):
    import torch
    import torch.distributed as dist

    rank, world, local = bench.init_replicas("gloo")
    cpu = torch.device("cpu")
    bench.barrier(world)
    # each rank "timed" a different duration: the job is as slow as its slowest replica
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, world, cpu)
    value = bench.replica_value(world, 12.0, 4, slowest)
    frames = bench.make_frames(TINY, rank, reference=True)
    digest = hashlib.sha256(b"".join(f[0].tobytes() for f in frames)).hexdigest()
    digests = [None] * world
    dist.all_gather_object(digests, digest)
    printed = io.StringIO()
    with contextlib.redirect_stdout(printed):
        bench.run_reference(types.SimpleNamespace(steps=1, warmup=0, gpus=world), TINY)
    bench.barrier(world)
    # what the reference arm brought into the process: no module of the product package and
    # none of its native libraries
    with open("/proc/self/maps") as f:
        maps = f.read()
    product = sorted(m for m in sys.modules if m == "climage_gb300" or m.startswith("climage_gb300."))
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"rank": rank, "world": world, "local": local, "slowest_ms": slowest, "value": value,
                   "digests": digests, "printed": printed.getvalue(), "product_modules": product,
                   "product_library_mapped": "libgls_cuda" in maps}, f)
    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1])
