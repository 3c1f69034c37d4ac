"""bench.py's reference arm runs on the CPU (the CPU restatement of the reference's path) and
prints one JSON line with the contract's keys; checked here on small bounded samples."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline",
        "e2e"}


@pytest.mark.parametrize("workload", ["explicit_bump_72k", "implicit_bump_72k"])
def test_reference_arm_prints_the_contract_line(workload):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", workload, "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert KEYS <= set(line)
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["cells"] == 72000  # the workload's own mesh


def _max_rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    q.put((rank, bench.max_over_ranks(10.0 + rank, dist)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    """The bench's timings are the maximum over ranks (replicas on N GPUs)."""
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_max_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 11.0, 1: 11.0}


def test_reference_arm_under_torchrun_prints_one_line():
    """Launched by torchrun with N ranks, only rank 0 runs the reference arm and prints."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                          "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                          "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                          "--impl", "reference", "--workload", "explicit_bump_72k", "--gpus", "2",
                          "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2


def test_explicit_fp64_work_uses_the_counted_flops():
    """The explicit line's FP64 work figure: the per-face constant is the counted Roe flux (add
    and mul) plus the five area products, and the per-cell-update figure follows from it."""
    sys.path.insert(0, ROOT)
    import bench
    from tests.test_flux_opcount import EXPECTED
    roe = EXPECTED["roe"]
    assert bench.FLOPS_PER_FACE_STAGE == roe["add"] + roe["mul"] + 5
    w = bench.explicit_fp64_work(72000, 148000, 1e8)
    per_cell = (72000 * (4 * bench.FLOPS_PER_CELL_STAGE + bench.FLOPS_PER_CELL_DT)
                + 148000 * 4 * bench.FLOPS_PER_FACE_STAGE) / 72000
    assert w["flops_per_cell_update"] == pytest.approx(per_cell)
    assert w["achieved_tflops"] == pytest.approx(1e8 * per_cell / 1e12)
