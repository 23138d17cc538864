"""bench.py --gpus N: N independent replicas, one process per GPU.  The path has
no data exchange between plumes; the only cross-rank operations are the
barrier around the timed region and the max / sum reductions of the timing.
Checked here with two gloo ranks on the CPU."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world)
    d.barrier()
    ms = 10.0 * (rank + 1)          # per-rank timed-region duration
    steps = 5 + rank                # per-rank steps
    ms_max = d.max(ms)
    total = d.sum(steps)
    d.barrier()
    # the reference arm: ranks other than 0 return at once without work
    class A:
        steps = 2
    rc = bench.run_reference(A(), rank, world) if rank != 0 else 0
    out.put((rank, ms_max, total, rc))
    d.td.destroy_process_group()


def test_two_replicas_reduce_timing_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms_max, total, rc in res:
        assert ms_max == 20.0          # whole-job time = the slowest rank
        assert total == 11.0           # units processed by all ranks
        assert rc == 0
    # value = all ranks' steps / slowest rank's time
    assert abs(res[0][2] / (res[0][1] / 1000.0) - 550.0) < 1e-9


def test_hyperplane_count_is_the_recurrence_length():
    """The sweep's hyperplane count in bench.py's roofline: the interior i+j+k
    planes of the MIC(0) recurrence at every grid of the benchmark sizes."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    sizes = {(32, 32, 32): 88, (48, 64, 48): 152, (64, 96, 64): 216, (96, 128, 96): 312,
             (128, 192, 128): 440, (256, 384, 256): 888}
    for res, want in sizes.items():
        assert bench.hyperplanes(res) == want
