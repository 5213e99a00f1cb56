"""Independent RIR work spread over ranks (one process per GPU).

Every RIR depends only on its room, source and receiver, so a multi-GPU run has
no exchange on the data path: rooms are dealt to ranks by estimated cost
(longest first, each to the least-loaded rank), every rank simulates its rooms
with one batched launch, and the results are gathered on the host.  A moving-source
trajectory is dealt by contiguous runs of its points: each rank filters its run, and
adjacent runs overlap only in the L - 1 samples past a run's end, which the host
gather adds up.  The only collectives are these gathers and the max-over-ranks of a
time.
"""
import math

import numpy as np


def room_cost(room, fs):
    """Work estimate of one room: windowed updates (RIRs x images x window) plus
    the samples written (tail and early part)."""
    m = len(np.asarray(room["pos_src"]).reshape(-1, 3)) * len(np.asarray(room["pos_rcv"]).reshape(-1, 3))
    n_img = int(np.prod(np.asarray(room["nb_img"]).reshape(3)))
    tw = round(8e-3 * fs)
    n_tot = math.ceil(room["Tmax"] * fs)
    return m * (n_img * tw + n_tot)


def partition(costs, world):
    """Longest-processing-time assignment: indices per rank, deterministic
    (ties by index).  Every index appears exactly once."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def _gpu_rooms(rooms, fs):
    """Default per-rank work: one batched launch, results as host arrays."""
    import torch
    from . import batch
    if not rooms:
        return []
    out, _ = batch.simulate_batch(rooms, fs)
    torch.cuda.synchronize()
    return batch.unpack(out.cpu().numpy(), rooms, fs)


def simulate_sharded(rooms, fs, simulate=None, group=None):
    """Simulate `rooms` over the ranks of `group` (torch.distributed, initialised).

    `simulate(rooms_subset, fs)` returns one array per room (default: the
    batched GPU call).  Every rank returns the full list in room order."""
    import torch.distributed as dist
    simulate = simulate or _gpu_rooms
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    mine = partition([room_cost(r, fs) for r in rooms], world)[rank]
    local = simulate([rooms[i] for i in mine], fs)
    pieces = [None] * world
    dist.all_gather_object(pieces, list(zip(mine, local)), group=group)
    result = [None] * len(rooms)
    for piece in pieces:
        for i, arr in piece:
            result[i] = arr
    return result


def trajectory_shards(n_pts, world):
    """Contiguous runs of trajectory points [p0, p1) per rank, as equal as the count
    allows (every point costs one convolution per receiver)."""
    bounds = [n_pts * k // world for k in range(world + 1)]
    return [(bounds[k], bounds[k + 1]) for k in range(world)]


def _gpu_trajectory(source_signal, RIRs, timestamps, fs):
    from .trajectory import simulate_trajectory
    return simulate_trajectory(source_signal, RIRs, timestamps, fs)


def simulate_trajectory_sharded(source_signal, RIRs, timestamps=None, fs=None, simulate=None, group=None):
    """simulateTrajectory (float64 [len(signal) + L - 1, R]) over the ranks of `group`
    (torch.distributed, initialised).  Rank k filters the points of its run [p0, p1):
    its slice of the signal, cut at the same samples as the whole call cuts it, with
    those points' RIRs, by `simulate(signal, RIRs, timestamps, fs)` (default: the GPU
    call); every rank returns the sum of all runs placed at their first samples."""
    import torch.distributed as dist
    from .trajectory import segment_bounds
    simulate = simulate or _gpu_trajectory
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    sig = np.asarray(source_signal)
    P, R, L = RIRs.shape
    w_ini = segment_bounds(len(sig), P, timestamps, fs)
    p0, p1 = trajectory_shards(P, world)[rank]
    piece = None
    if p1 > p0:
        # timestamps in samples (fs = 1): the run's cut points exactly
        local = simulate(sig[w_ini[p0]:w_ini[p1]], RIRs[p0:p1],
                         (w_ini[p0:p1] - w_ini[p0]).astype(np.float64), 1.0)
        piece = (int(w_ini[p0]), np.asarray(local, dtype=np.float64))
    pieces = [None] * world
    dist.all_gather_object(pieces, piece, group=group)
    out = np.zeros((len(sig) + L - 1, R), dtype=np.float64)
    for pc in pieces:
        if pc is not None:
            off, a = pc
            out[off:off + a.shape[0]] += a
    return out


def max_over_ranks(value, group=None):
    """Largest `value` over the ranks (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" \
        else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
