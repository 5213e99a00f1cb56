"""Polar-pattern sweep: the scene of the reference's polar-plot example
(examples/polar_plots.py:113-156 of gpuRIR) -- a 16 x 8 x 3 m room, beta 0.1 on
every wall, 44.1 kHz, T60 0.21 s with the diffuse model from 15 dB and the RIR
to 60 dB, the source at (4, 4, 1.7) turned through 360 orientations in the
horizontal plane, an omni receiver at (10, 4, 2) -- for every source pattern.

Each orientation's RIR is compared with the FP64 oracle (early part relative L2
<= 1e-5), and so is the curve the example plots: the largest |RIR| sample per
orientation (relative error <= 1e-5 at every angle).  The curve also follows the
pattern's own gain: its peak is the direct path, whose amplitude is
gain(cos theta) / (4 pi d), so peak / max(peak) matches the gain normalised the
same way to 1e-2 wherever the gain is above half its maximum (there the direct
path is the peak sample; the weak reflections add the rest).
"""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu

PARTITIONS = 360
GAIN = {"omni": lambda c: np.ones_like(c), "homni": lambda c: (c > 0).astype(float),
        "card": lambda c: 0.5 + 0.5 * c, "hypcard": lambda c: 0.25 + 0.75 * c,
        "subcard": lambda c: 0.75 + 0.25 * c, "bidir": lambda c: c}


@pytest.mark.parametrize("pattern", ["omni", "homni", "card", "hypcard", "subcard", "bidir"])
def test_polar_sweep(built, pattern):
    import gpurir_gb300 as G
    room = [16.0, 8.0, 3.0]
    rad = np.arange(PARTITIONS) * (2 * np.pi / PARTITIONS)
    orv = np.stack([np.cos(rad), np.sin(rad), np.zeros_like(rad)], axis=1).astype(np.float32)
    ps = np.tile(np.array([[4.0, 4.0, 1.7]], np.float32), (PARTITIONS, 1))
    pr = np.array([[10.0, 4.0, 2.0]], np.float32)
    T60, fs, beta = 0.21, 44100.0, [0.1] * 6
    Tdiff = G.att2t_SabineEstimator(15.0, T60)
    Tmax = G.att2t_SabineEstimator(60.0, T60)
    nb = G.t2n(Tdiff, room)
    G.seed(5)
    rir = G.simulateRIR(room, beta, ps, pr, nb, Tmax, fs, Tdiff=Tdiff, spkr_pattern=pattern, orV_src=orv,
                        mic_pattern="omni")
    ref, parts = oracle.simulate_rir(room, beta, ps, pr, nb, Tmax, fs, Tdiff, pattern, "omni", orv, None,
                                     seed=5, offset=0, return_parts=True)
    n = parts["n_ism"]
    assert rel_l2(rir[..., :n], ref[..., :n]) <= 1e-5
    # the example's curve: the largest |sample| per orientation (in the early part here: the
    # tail's noise is not the reference's stream)
    early_peak = np.abs(rir[:, 0, :n]).max(axis=1).astype(np.float64)
    peak_ref = np.abs(ref[:, 0, :n]).max(axis=1)
    assert np.all(np.abs(early_peak - peak_ref) <= 1e-5 * peak_ref.max())
    # the shape of the pattern: cos theta between the orientation and the direction to the receiver
    d = pr[0].astype(np.float64) - ps[0]
    cos_t = orv.astype(np.float64) @ (d / np.linalg.norm(d))
    g = np.abs(GAIN[pattern](cos_t))
    strong = g >= 0.5 * g.max()
    assert np.abs(early_peak[strong] / early_peak.max() - g[strong] / g.max()).max() <= 1e-2
