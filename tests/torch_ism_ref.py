"""FP64, differentiable torch transcription of the ISM early part (test infrastructure).

Same formulas as oracle/ism_oracle.c (image bookkeeping src/gpuRIR_cuda.cu:336-353,
directivity :132-147, windowed sinc :110-121), vectorised over the image grid so
torch.autograd gives FP64 gradients with respect to beta, positions and
orientations.  Used to check the CUDA adjoint kernel.
"""
import math

import numpy as np
import torch


def _axis(N):
    k = np.arange(N) - N // 2
    clust = np.ceil(k / 2.0).astype(np.int64)
    refl = np.abs(np.fmod(k, 2)).astype(np.int64)
    return clust, refl


def _gain(c, pattern):
    if pattern == "homni":
        return (c > 0).to(c.dtype)
    return {"card": 0.5 + 0.5 * c, "hypcard": 0.25 + 0.75 * c, "subcard": 0.75 + 0.25 * c,
            "bidir": c}[pattern]


def early_part(room_sz, beta, pos_src, pos_rcv, nb_img, n_ism, fs, c=343.0, spkr="omni", mic="omni",
               orV_src=None, orV_rcv=None):
    """h [M_src, M_rcv, n_ism] float64; beta [6], pos_* [M, 3], orV_* [M, 3] torch float64."""
    dev = beta.device
    L = torch.as_tensor(np.asarray(room_sz, dtype=np.float32).astype(np.float64), device=dev)
    cl = [torch.as_tensor(_axis(n)[0], device=dev) for n in nb_img]
    rf = [torch.as_tensor(_axis(n)[1], device=dev) for n in nb_img]
    grids = torch.meshgrid(*[torch.arange(n, device=dev) for n in nb_img], indexing="ij")
    C = torch.stack([cl[d][grids[d]].reshape(-1) for d in range(3)], 1)      # [N, 3]
    Rf = torch.stack([rf[d][grids[d]].reshape(-1) for d in range(3)], 1)
    sgn = (1 - 2 * Rf).to(torch.float64)
    att = torch.ones(C.shape[0], dtype=torch.float64, device=dev)
    for d in range(3):
        att = att * (-beta[2 * d]) ** (C[:, d] - Rf[:, d]).abs().to(torch.float64) * \
            (-beta[2 * d + 1]) ** C[:, d].abs().to(torch.float64)
    Tw = int(round(float(np.float32(8e-3) * np.float32(fs))))
    H = Tw / 2.0
    K = float(np.float32(fs)) / float(np.float32(c))
    out = []
    t = torch.arange(n_ism, dtype=torch.float64, device=dev)
    for s in range(pos_src.shape[0]):
        row = []
        img = 2 * C.to(torch.float64) * L + sgn * pos_src[s]                  # [N, 3]
        for r in range(pos_rcv.shape[0]):
            v = img - pos_rcv[r]
            dist = torch.sqrt((v * v).sum(1))
            amp = att / (4 * math.pi * dist)
            if spkr != "omni":
                o = orV_src[s]
                cs = -(sgn * o * v).sum(1) / dist / torch.sqrt((o * o).sum())
                amp = amp * _gain(cs, spkr)
            if mic != "omni":
                o = orV_rcv[r]
                cm = (o * v).sum(1) / dist / torch.sqrt((o * o).sum())
                amp = amp * _gain(cm, mic)
            tau = dist * K
            x = t[None, :] - tau[:, None]                                      # [N, T]
            w = torch.where(x.abs() < H, 0.5 * (1 + torch.cos(2 * math.pi * x / Tw)),
                            torch.zeros_like(x))
            h = (amp[:, None] * w * torch.sinc(x)).sum(0)
            row.append(h)
        out.append(torch.stack(row))
    return torch.stack(out)
