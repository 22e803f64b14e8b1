"""Trial sharding over two gloo ranks on the CPU: the union of the ranks'
candidate lists equals the single-process list.  The per-rank work is the
FP64 oracle on a small configuration (no GPU)."""
import os
import socket

import numpy as np
import pytest

from gpu_accelsearch_gb300.shard import shard_trials

torch = pytest.importorskip("torch")


def test_shard_cover_and_balance():
    costs = [1 << 20, 1 << 21, 1 << 22, 3 << 20, 1 << 20, 1 << 22, 1 << 21]
    for world in (1, 2, 3, 4):
        parts = [shard_trials(len(costs), r, world, costs) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
        rr = [shard_trials(len(costs), r, world) for r in range(world)]
        assert sorted(i for p in rr for i in p) == list(range(len(costs)))


def _trials():
    from gpu_accelsearch_gb300.synth import synth_series
    from oracle import oracle as O
    out = []
    for k in range(3):
        n = 1 << 15
        x = synth_series(n, seed=300 + k, signals=[(0.3, 2000.25 + 500 * k, 10.0)])
        spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
        out.append(O.deredden(spec))
    return out


def _search(idx, trials):
    from oracle import oracle as O
    orc = O.Oracle(50, 2, 1914)
    cuts = np.array([O.power_cut(4.0, 1 << s) for s in range(orc.nstages)])
    res = []
    for local_i, t in enumerate(idx):
        w = trials[t]
        nsteps = O.step_count(w.size, 2, 1914)
        c, _, _ = orc.run_steps(w, 2, 0, nsteps, powcut=cuts, nthreads=1)
        arr = np.zeros(len(c), dtype=[("trial", "i4"), ("step", "i4"), ("r", "f8"), ("z", "f8"),
                                      ("numharm", "i4"), ("power", "f4"), ("sigma", "f4")])
        arr["trial"] = local_i
        arr["step"] = c["step"]
        arr["r"] = 2 + c["step"] * 957 + 0.5 * c["ridx"]
        arr["z"] = -50 + 2 * c["zidx"]
        arr["numharm"] = c["numharm"]
        arr["power"] = c["power"]
        res.append(arr)
    orc.close()
    return np.concatenate(res) if res else None


def _rank(rank, world, port, q):
    import torch.distributed as dist
    from gpu_accelsearch_gb300.shard import gather_candidates, shard_trials
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    trials = _trials()
    idx = shard_trials(len(trials), rank, world, [t.size for t in trials])
    local = _search(idx, trials)
    allc = gather_candidates(local, idx)
    if rank == 0:
        q.put(allc.tobytes())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_union_equals_single_process():
    import torch.multiprocessing as mp
    from gpu_accelsearch_gb300.shard import gather_candidates
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    trials = _trials()
    single = gather_candidates(_search([0, 1, 2], trials), [0, 1, 2])
    assert len(single) > 0
    assert got == single.tobytes()
