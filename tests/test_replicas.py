"""The multi-GPU path (replicas: no data-path collective) run as 2 gloo ranks on CPU.

Each rank simulates the rooms the cost partition gives it (here with the oracle,
standing in for the GPU call), the host gather reassembles them in room order, and
the job time is the max over ranks."""
import os
import socket

import numpy as np
import pytest

from gpurir_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rooms():
    rng = np.random.default_rng(5)
    rooms = []
    for i in range(7):
        room = rng.uniform([3, 3, 2.5], [6, 5, 3.5])
        ms, mr = int(rng.integers(1, 3)), int(rng.integers(1, 4))
        rooms.append(dict(room_sz=room.astype(np.float32), beta=rng.uniform(0.6, 0.9, 6).astype(np.float32),
                          pos_src=(0.5 + rng.random((ms, 3)) * (room - 1)).astype(np.float32),
                          pos_rcv=(0.5 + rng.random((mr, 3)) * (room - 1)).astype(np.float32),
                          nb_img=[int(x) for x in rng.integers(3, 8, 3)], Tmax=0.02 + 0.01 * i,
                          Tdiff=0.02 + 0.01 * i))
    return rooms


def _oracle_rooms(rooms, fs):
    import oracle
    return [oracle.simulate_rir(r["room_sz"], r["beta"], r["pos_src"], r["pos_rcv"], r["nb_img"],
                                r["Tmax"], fs, Tdiff=r["Tdiff"]) for r in rooms]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rooms = _rooms()
        res = replicas.simulate_sharded(rooms, 16000.0, simulate=_oracle_rooms)
        t = replicas.max_over_ranks(1.5 + rank)          # rank 1 is the slow one
        np.savez(os.path.join(out_dir, "rank%d.npz" % rank), t=t,
                 **{"r%d" % i: a for i, a in enumerate(res)})
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_partition_covers_every_room_once_and_balances():
    costs = [9, 1, 4, 4, 7, 2, 2, 8]
    parts = replicas.partition(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert replicas.partition(costs, 3) == parts            # deterministic
    assert replicas.partition(costs, 1) == [list(range(len(costs)))]


def test_two_gloo_ranks_gather_every_room(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    want = _oracle_rooms(_rooms(), 16000.0)
    for rank in range(world):
        z = np.load(tmp_path / ("rank%d.npz" % rank))
        assert float(z["t"]) == 2.5
        for i, w in enumerate(want):
            assert np.array_equal(z["r%d" % i], w)


def _traj_case(custom):
    rng = np.random.default_rng(6)
    sig = rng.standard_normal(3001).astype(np.float32)
    rirs = (0.1 * rng.standard_normal((9, 2, 50))).astype(np.float32)
    if not custom:
        return sig, rirs, None, None
    # uneven segments, timestamps in seconds at 10 kHz
    ts = np.array([0.0, 0.013, 0.05, 0.061, 0.1, 0.17, 0.2, 0.23, 0.29])
    return sig, rirs, ts, 10000.0


def _oracle_trajectory(sig, rirs, ts, fs):
    import oracle
    return oracle.trajectory(sig, rirs, ts, fs)


def _traj_worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        for custom in (False, True):
            sig, rirs, ts, fs = _traj_case(custom)
            res = replicas.simulate_trajectory_sharded(sig, rirs, ts, fs, simulate=_oracle_trajectory)
            np.save(os.path.join(out_dir, "traj%d_%d.npy" % (rank, custom)), res)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_trajectory_shards_are_contiguous_runs():
    for n_pts, world in [(9, 2), (400, 8), (2, 3), (1, 1)]:
        runs = replicas.trajectory_shards(n_pts, world)
        assert len(runs) == world and runs[0][0] == 0 and runs[-1][1] == n_pts
        assert all(a[1] == b[0] for a, b in zip(runs, runs[1:]))
        sizes = [p1 - p0 for p0, p1 in runs]
        assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_overlap_add_a_trajectory(tmp_path):
    """Each rank filters a contiguous run of trajectory points (the oracle standing in for
    the GPU call); the gathered runs, overlapping in L - 1 samples at the run edge, equal
    the unsharded overlap-add, with equal and with custom segments."""
    import oracle
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_traj_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    for custom in (False, True):
        sig, rirs, ts, fs = _traj_case(custom)
        want = oracle.trajectory(sig, rirs, ts, fs)
        for rank in range(world):
            got = np.load(tmp_path / ("traj%d_%d.npy" % (rank, custom)))
            assert got.shape == want.shape
            assert np.allclose(got, want, rtol=1e-12, atol=1e-12)
