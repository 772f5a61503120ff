"""Failure detection on the host (no GPU involved): corrupt and truncated input files are
reported with a clear error instead of wrong results, and a replica rank that dies is
noticed by the surviving rank through the process group's timeout."""
import datetime
import os
import socket
import subprocess

import numpy as np
import pytest

from ses3d_gb300 import formats as F
from ses3d_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "ses3d_gb300", "ses3d_gpu_main")


def tree(tmp_path, procs=(2, 1, 1)):
    p = synth.make_problem("tiny", nt=5, seed=91, n_el=(6, 5, 4))
    root = str(tmp_path / "tree")
    synth.write_problem(p, root, procs=procs)
    return p, root


def stitch(root, out):
    return subprocess.run([DRIVER, "--main", os.path.join(root, "MAIN"), "--stitch-model", out],
                          capture_output=True, text=True, timeout=120)


def test_truncated_record_is_reported_by_the_python_reader(tmp_path):
    path = str(tmp_path / "rec")
    F.write_records(path, [np.arange(100, dtype=np.float32), np.arange(50, dtype=np.float32)])
    data = open(path, "rb").read()
    open(path, "wb").write(data[:-20])
    with pytest.raises(ValueError, match="truncated"):
        F.read_records(path)


def test_driver_reports_truncated_model_file(native, tmp_path):
    p, root = tree(tmp_path)
    f = os.path.join(root, "MODELS", "MODELS", "mu1")
    data = open(f, "rb").read()
    open(f, "wb").write(data[: len(data) // 2])
    res = stitch(root, str(tmp_path / "out"))
    assert res.returncode == 1 and "truncated record" in res.stderr and "mu1" in res.stderr


def test_driver_reports_missing_model_file(native, tmp_path):
    p, root = tree(tmp_path)
    os.remove(os.path.join(root, "MODELS", "MODELS", "lambda0"))
    res = stitch(root, str(tmp_path / "out"))
    assert res.returncode == 1 and "cannot open" in res.stderr and "lambda0" in res.stderr


def test_driver_reports_overlapping_boxes(native, tmp_path):
    p, root = tree(tmp_path)
    bf = os.path.join(root, "MODELS", "MODELS", "boxfile")
    boxes = F.read_boxfile(bf)
    boxes[1].nx_min -= 1          # box 2 now starts inside box 1
    F.write_boxfile(bf, boxes, 2, 1, 1)
    res = stitch(root, str(tmp_path / "out"))
    assert res.returncode == 1 and "overlap" in res.stderr


def test_driver_reports_missing_event_before_touching_the_gpu(native, tmp_path):
    p, root = tree(tmp_path, procs=(1, 1, 1))
    os.remove(os.path.join(root, "INPUT", "event_" + p.events[0].name))
    res = subprocess.run([DRIVER, "--main", os.path.join(root, "MAIN")], capture_output=True, text=True, timeout=120)
    assert res.returncode == 1 and "event_" in res.stderr and "no CUDA device" not in res.stderr


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, port, q):
    import sys
    sys.path[:0] = [ROOT]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      OMP_NUM_THREADS="1")
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=2, timeout=datetime.timedelta(seconds=5))
    from ses3d_gb300 import replicas
    if rank == 1:
        os._exit(3)               # the replica dies between steps, before the kernel sum
    try:
        replicas.sum_over_ranks([np.ones(8)])
        q.put((rank, "no error"))
    except Exception as e:        # the survivor learns of it from the collective
        q.put((rank, "error: " + type(e).__name__))


def test_surviving_replica_detects_a_dead_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    rank, msg = q.get(timeout=120)
    for pr in procs:
        pr.join(timeout=60)
    assert rank == 0 and msg.startswith("error"), msg
    assert procs[1].exitcode == 3
