"""Seeded synthetic scenes of the five benchmark workloads, and work counters.

Each scene is a dict of numpy arrays / scalars with simulateRIR's argument
names.  No dataset is involved; sizes, distributions and seeds are fixed here.

  plain_room       1 source x 2 receivers, room 3 x 4 x 2.5 m, full ISM 0.5 s,
                   nb_img [11, 9, 13], beta 0.85, omni (seed 0)
  mic_array        64 omni sources x 32 cardioid receivers on a 0.2 m sphere,
                   room 6 x 5 x 3 m, Sabine beta at T60 = 1 s, Tdiff 0.3 s,
                   Tmax 1 s, nb_img [12, 14, 24], Gaussian tail (seed 1)
  batched_rooms    512 rooms of uneven size / T60 / source and receiver counts
                   (seed 2)
  inverse_problem  16 rooms 5 x 4 x 3 m, 4 sources x 8 hypercardioid receivers,
                   0.4 s full ISM, nb_img [9, 11, 13] (seed 3)
  trajectory       one source moving over 400 points, 8-mic linear array,
                   room 8 x 6 x 3 m, T60 0.8 s, 10 s white-noise signal (seed 4)
"""
import math

import numpy as np


def _inside(rng, n, room, margin):
    room = np.asarray(room, dtype=np.float64)
    return (margin + rng.random((n, 3)) * (room - 2 * margin)).astype(np.float32)


def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def plain_room():
    rng = np.random.default_rng(0)
    room = [3.0, 4.0, 2.5]
    return dict(room_sz=room, beta=[0.85] * 6, pos_src=_inside(rng, 1, room, 0.5),
                pos_rcv=_inside(rng, 2, room, 0.5), nb_img=[11, 9, 13], Tmax=0.5, fs=16000.0,
                Tdiff=0.5, spkr_pattern="omni", mic_pattern="omni", orV_src=None, orV_rcv=None,
                c=343.0, noise="logistic")


def mic_array():
    from . import beta_SabineEstimation
    rng = np.random.default_rng(1)
    room = [6.0, 5.0, 3.0]
    ps = _inside(rng, 64, room, 0.5)
    v = rng.standard_normal((32, 3))
    pr = (np.asarray(room) / 2 + 0.2 * v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    return dict(room_sz=room, beta=beta_SabineEstimation(room, 1.0), pos_src=ps, pos_rcv=pr,
                nb_img=[12, 14, 24], Tmax=1.0, fs=16000.0, Tdiff=0.3, spkr_pattern="omni",
                mic_pattern="card", orV_src=None, orV_rcv=_unit(rng, 32), c=343.0, noise="gaussian")


def batched_rooms(n_rooms=512, c=343.0):
    from . import beta_SabineEstimation
    rng = np.random.default_rng(2)
    dims = np.stack([rng.uniform(3, 10, n_rooms), rng.uniform(3, 8, n_rooms),
                     rng.uniform(2.5, 4.5, n_rooms)], axis=1)
    t60 = rng.uniform(0.2, 1.2, n_rooms)
    # beta per room by the reference's own estimator (scipy L-BFGS-B, gpuRIR/__init__.py:22-54)
    betas = [beta_SabineEstimation(dims[i], t60[i]) for i in range(n_rooms)]
    rooms = []
    for i in range(n_rooms):
        tdiff = 0.4 * t60[i]
        nb = [int(math.ceil(2 * c * tdiff / d)) for d in dims[i]]
        ns = int(rng.integers(1, 5))
        nr = int(rng.integers(2, 9))
        rooms.append(dict(room_sz=dims[i].astype(np.float32), beta=betas[i],
                          pos_src=_inside(rng, ns, dims[i], 0.3), pos_rcv=_inside(rng, nr, dims[i], 0.3),
                          nb_img=nb, Tmax=float(t60[i]), Tdiff=float(tdiff), fs=16000.0,
                          spkr_pattern="omni", mic_pattern="omni", orV_src=None, orV_rcv=None, c=c))
    return rooms


def inverse_problem():
    rng = np.random.default_rng(3)
    room = [5.0, 4.0, 3.0]
    rooms = []
    for _ in range(16):
        rooms.append(dict(room_sz=room, beta=rng.uniform(0.6, 0.95, 6).astype(np.float32),
                          pos_src=_inside(rng, 4, room, 0.5), pos_rcv=_inside(rng, 8, room, 0.5),
                          orV_rcv=_unit(rng, 8), orV_src=None, spkr_pattern="omni",
                          mic_pattern="hypcard", nb_img=[9, 11, 13], Tmax=0.4, Tdiff=0.4,
                          fs=16000.0, c=343.0))
    return rooms


def trajectory():
    from . import beta_SabineEstimation
    rng = np.random.default_rng(4)
    room = [8.0, 6.0, 3.0]
    n_pts = 400
    t = np.linspace(0.0, 1.0, n_pts)[:, None]
    traj = (np.array([1.0, 1.0, 1.5]) + t * np.array([6.0, 4.0, 0.0])).astype(np.float32)
    mics = np.stack([4.0 + 0.05 * (np.arange(8) - 3.5), np.full(8, 3.0), np.full(8, 1.2)],
                    axis=1).astype(np.float32)
    signal = rng.standard_normal(160000).astype(np.float32)
    return dict(room_sz=room, beta=beta_SabineEstimation(room, 0.8), pos_src=traj, pos_rcv=mics,
                nb_img=[8, 10, 28], Tmax=0.8, Tdiff=0.25, fs=16000.0, spkr_pattern="omni",
                mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0, signal=signal)


def n_samples(T, fs):
    """ceil(T*fs) in float32, rounded up to even (the simulator's lengths)."""
    n = int(np.ceil(np.float32(T) * np.float32(fs)))
    return n + n % 2


def windowed_updates(scene, chunk=1 << 22):
    """Number of (RIR, image, t) triples with 0 <= t < nISM and |t - tau| < Tw/2,
    the unit of work of the sinc accumulation, counted in FP64 numpy.
    Also returns the brute-force count M * N * nISM that gpuRIR evaluates."""
    room = np.asarray(scene["room_sz"], dtype=np.float64)
    nb = np.asarray(scene["nb_img"], dtype=np.int64)
    fs, c = float(np.float32(scene["fs"])), float(np.float32(scene.get("c", 343.0)))
    tdiff = scene.get("Tdiff") or scene["Tmax"]
    n_ism = n_samples(tdiff, fs)
    H = int(round(float(np.float32(8e-3) * np.float32(fs)))) / 2.0
    ps = np.asarray(scene["pos_src"], dtype=np.float64)
    pr = np.asarray(scene["pos_rcv"], dtype=np.float64)
    axes = []
    for d in range(3):
        k = np.arange(nb[d]) - nb[d] // 2
        cl = np.ceil(k / 2.0)
        r = np.abs(np.fmod(k, 2))
        axes.append((2 * cl * room[d], 1 - 2 * r))
    off = [a[0] for a in axes]
    sg = [a[1] for a in axes]
    total = 0
    for s in ps:
        comp = [off[d][:, None] + sg[d][:, None] * s[d] - pr[None, :, d] for d in range(3)]
        # squared distance over the image grid, per receiver
        d2 = (comp[0][:, None, None, :] ** 2 + comp[1][None, :, None, :] ** 2 +
              comp[2][None, None, :, :] ** 2)
        tau = np.sqrt(d2) * (fs / c)
        lo = np.maximum(np.floor(tau - H) + 1, 0)
        hi = np.minimum(np.ceil(tau + H) - 1, n_ism - 1)
        total += int(np.maximum(hi - lo + 1, 0).sum())
    M = ps.shape[0] * pr.shape[0]
    return total, M * int(np.prod(nb)) * n_ism


def windowed_updates_torch(scene, device="cuda"):
    """windowed_updates computed with torch (FP64) on `device`, for large scenes."""
    import torch
    room = torch.tensor(np.asarray(scene["room_sz"], dtype=np.float32).astype(np.float64), device=device)
    nb = [int(x) for x in np.asarray(scene["nb_img"]).reshape(3)]
    fs = float(np.float32(scene["fs"]))
    c = float(np.float32(scene.get("c", 343.0)))
    tdiff = scene.get("Tdiff") or scene["Tmax"]
    n_ism = n_samples(tdiff, fs)
    H = int(round(float(np.float32(8e-3) * np.float32(fs)))) / 2.0
    ps = torch.tensor(np.asarray(scene["pos_src"], dtype=np.float64), device=device).reshape(-1, 3)
    pr = torch.tensor(np.asarray(scene["pos_rcv"], dtype=np.float64), device=device).reshape(-1, 3)
    off, sg = [], []
    for d in range(3):
        k = torch.arange(nb[d], device=device, dtype=torch.float64) - (nb[d] // 2)
        cl = torch.ceil(k / 2.0)
        r = torch.fmod(k, 2).abs()
        off.append(2 * cl * room[d])
        sg.append(1 - 2 * r)
    total = 0
    for s in ps:
        for rv in pr:
            comp = [off[d] + sg[d] * s[d] - rv[d] for d in range(3)]
            d2 = (comp[0][:, None, None] ** 2 + comp[1][None, :, None] ** 2 +
                  comp[2][None, None, :] ** 2)
            tau = torch.sqrt(d2) * (fs / c)
            lo = torch.clamp(torch.floor(tau - H) + 1, min=0)
            hi = torch.clamp(torch.ceil(tau + H) - 1, max=n_ism - 1)
            total += int(torch.clamp(hi - lo + 1, min=0).sum().item())
    return total
