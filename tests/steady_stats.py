"""Steady-state statistics of the ch3/ver2 sphere run (ch3/ver2/Main.cpp:18-80:
21x21x41 nodes on [-0.1,0.1]^2 x [0,0.4] m, a cold O+ beam at 7 km/s and
1e10 m^-3 from the z = 0 face, a sphere of radius 0.05 m at -100 V): the
reductions of batch-mean density and potential fields to profiles, shared by
the golden generator (applied to the reference's own run) and the GPU test.

Fields are flat in (k, j, i) order, nodes (21, 21, 41) in (i, j, k).
"""
import numpy as np

NI, NJ, NK = 21, 21, 41
STEPS, DT, MPW0 = 600, 1e-7, 50.0
AVG = (200, 40, 10)         # first time step, steps per batch, batches
KEYS = ("axial", "wake", "radial", "phi_axis")
C = 10                      # the axis x = y = 0
WAKE_K = slice(25, 36)      # z in [0.25, 0.35] m, behind the sphere (z <= 0.2)


def profiles(den, phi):
    """1-D profiles of one (batch-mean) density and potential field."""
    d = np.asarray(den).reshape(NK, NJ, NI)
    p = np.asarray(phi).reshape(NK, NJ, NI)
    ii, jj = np.meshgrid(np.arange(NI), np.arange(NJ))
    ring = np.maximum(np.abs(ii - C), np.abs(jj - C))
    dw = d[WAKE_K].mean(axis=0)
    return {
        "axial": d.mean(axis=(1, 2)),                      # plane mean per k
        "wake": d[:, C - 1:C + 2, C - 1:C + 2].mean(axis=(1, 2)),  # near-axis per k
        "radial": np.array([dw[ring == r].mean() for r in range(C + 1)]),
        "phi_axis": p[:, C, C].copy(),
    }


def batch_profiles(den_batches, phi_batches):
    """The profiles of each batch-mean field, stacked: key -> (batches, n)."""
    per = [profiles(d, p) for d, p in zip(den_batches, phi_batches)]
    return {key: np.stack([q[key] for q in per]) for key in per[0]}


def batch_stats(stacked):
    """Mean and standard error (method of batch means) of each stacked
    profile or total."""
    out = {}
    for key, a in stacked.items():
        out[key] = a.mean(axis=0)
        out[key + "_se"] = a.std(axis=0, ddof=1) / np.sqrt(a.shape[0])
    return out


def batch_index(ts):
    """The batch that time step ts (0-based, as World::getTs) falls in, or -1."""
    if ts < AVG[0] or (ts - AVG[0]) // AVG[1] >= AVG[2]:
        return -1
    return (ts - AVG[0]) // AVG[1]


def pooled(per_seed):
    """Mean and standard error over runs with independent seeds, each given
    as the output of batch_stats."""
    n = len(per_seed)
    out = {}
    for key in per_seed[0]:
        if key.endswith("_se"):
            out[key] = np.sqrt(sum(r[key] ** 2 for r in per_seed)) / n
        else:
            out[key] = sum(r[key] for r in per_seed) / n
    return out


def z_scores(a, b, key):
    """Differences of a profile between two estimates in units of their
    combined standard error, and the differences where that error is zero
    (nodes inside the sphere, fixed potential)."""
    d = a[key] - b[key]
    s = np.sqrt(a[key + "_se"] ** 2 + b[key + "_se"] ** 2)
    m = s > 0
    return d[m] / s[m], d[~m]
