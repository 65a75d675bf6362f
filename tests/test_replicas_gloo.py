"""The N>1 form of the bench on the CPU: two processes over gloo (world size 2) run bench.py's
replica helpers.  The pipeline does not shard, so each rank converts its own frames with no
collective on the data path; what crosses ranks is the barrier around the timed region and
the max-over-ranks reduction of its duration, and only rank 0 runs and prints the
reference arm."""
import json
import os
import socket
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.fixture(scope="module")
def ranks(tmp_path_factory):
    out = tmp_path_factory.mktemp("replicas")
    port = str(free_port())
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, os.path.join(HERE, "replica_worker.py"), str(out)],
                                      cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                      text=True))
    logs = []
    try:
        for p in procs:
            logs.append(p.communicate(timeout=240)[0])
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
                p.wait()
    for r, (p, log) in enumerate(zip(procs, logs)):
        assert p.returncode == 0, "rank %d exited %s:\n%s" % (r, p.returncode, log[-3000:])
    res = []
    for r in range(2):
        with open(out / ("rank%d.json" % r)) as f:
            res.append(json.load(f))
    return res


def test_ranks_read_their_environment(ranks):
    assert [(x["rank"], x["world"], x["local"]) for x in ranks] == [(0, 2, 0), (1, 2, 1)]


def test_time_is_the_slowest_rank(ranks):
    assert [x["slowest_ms"] for x in ranks] == [15.0, 15.0]
    # 2 ranks x 4 steps x 12 Mpx in 15 ms
    assert ranks[0]["value"] == pytest.approx(2 * 4 * 12.0 / 15e-3)
    assert ranks[1]["value"] == ranks[0]["value"]


def test_each_rank_converts_its_own_frames(ranks):
    assert ranks[0]["digests"] == ranks[1]["digests"]
    assert len(set(ranks[0]["digests"])) == 2


def test_reference_arm_runs_on_rank_zero_only(ranks):
    assert ranks[1]["printed"] == ""
    lines = [l for l in ranks[0]["printed"].splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["n_gpus"] == 2
    assert line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_loads_nothing_of_the_product(ranks):
    """The reference arm (and the frames it converts) must not run or even map the product: no
    module of climage_gb300 imported, libgls_cuda.so not mapped."""
    for x in ranks:
        assert x["product_modules"] == []
        assert not x["product_library_mapped"]


def test_reference_arm_times_the_gpu_arms_workload(ranks):
    """Both arms describe the workload with the same config dict; each reference step
    converts every frame of the workload (three here, one per noise level)."""
    line = json.loads(ranks[0]["printed"].strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    import bench
    import replica_worker

    assert line["config"] == bench.workload_config(replica_worker.TINY, 2)
    assert line["config"]["frames_per_step"] == 3


def test_bench_starts_its_own_replicas(tmp_path):
    """bench.py --gpus 2 outside a launcher starts two ranks itself (torch.distributed.run on
    127.0.0.1); with --cpu-replicas each rank converts its own frames with the oracle over
    gloo and rank 0 prints the one check line."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR",
                                                             "MASTER_PORT")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--cpu-replicas", "--steps",
                        "1", "--warmup", "0"], cwd=str(tmp_path), env=env, capture_output=True, text=True,
                       timeout=240)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-3000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["check"] == "cpu-replicas" and line["n_ranks"] == 2
    assert len(set(line["digests"])) == 2  # each rank converted frames of its own
    assert line["config"]["parallelism"] == "replicas"


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(7.5, 1, None) == 7.5
    assert bench.replica_value(1, 12.0, 4, 15.0) == pytest.approx(4 * 12.0 / 15e-3)
