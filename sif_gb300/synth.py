"""Seeded synthetic inputs for the exodus path: Zel'dovich-displaced lattices.

The reference has no generator and the workloads name no public dataset, so
every benchmark and test box is made here:

- lattice q = (i + 1/2) L/N per axis, N^3 particles in a periodic box of side L;
- displacement psi_k = i k / k^2 delta_k, with delta_k a Gaussian random field
  of power P(k) = A k^-1 exp(-(k * 2 Mpc/h)^2) on the N^3 lattice;
- A fixed so that the rms of |psi| (3-D) is ``rms_disp``;
- x = q + psi(q) wrapped into [0, L), stored float32.

White noise comes from ``numpy.random.default_rng(seed)`` (bit-stable across
machines); the transforms run in float64, on the GPU through torch when asked
(the 512^3 and 1024^3 boxes), else in numpy. Positions agree across backends
and machines to float32 rounding of the displacement, not to the bit, so
parity fixtures store the positions themselves.

Also here: the radius ladder the workloads use, ``ladder(R, 6R, 0.10)``,
which is sif-exodus's ``ladder()`` helper (bin/sif-exodus/config.c:1853-1874).
"""
import math

import numpy as np

# The workloads: particles per side, box side, rms displacement, seed,
# smoothing radius R (the bottom rung), mesh cell size, threshold.
WORKLOADS = {
    "A": dict(n=128, box=500.0, rms_disp=4.0, seed=1001, radius=5.0, mesh_cell=10.0,
              threshold=-0.8),
    "B": dict(n=512, box=1000.0, rms_disp=5.0, seed=1002, radius=4.0, mesh_cell=8.0,
              threshold=-0.8),
    "C": dict(n=1024, box=2000.0, rms_disp=4.0, seed=1003, radius=5.0, mesh_cell=None,
              threshold=-0.8),
    "E": dict(n=256, box=500.0, rms_disp=4.0, seed=1005, radius=5.0, mesh_cell=10.0,
              threshold=-0.8),
}


def ladder(r_min, r_max, step):
    """r_min, r_min (1 + step), ... up to r_max, as sif-exodus's ladder()."""
    ratio = 1.0 + step
    count = int(math.floor(math.log(r_max / r_min) / math.log(ratio) + 1e-9) + 1.0)
    return np.array([r_min * ratio ** i for i in range(count)], dtype=np.float64)


def workload_radii(name):
    w = WORKLOADS[name]
    return ladder(w["radius"], 6.0 * w["radius"], 0.10).astype(np.float32)


def _kgrid(n, box, xp):
    kf = 2.0 * math.pi / box
    k1 = xp.fft.fftfreq(n, d=1.0 / n) * kf
    kz = xp.fft.rfftfreq(n, d=1.0 / n) * kf
    return k1, kz


def zeldovich(n, box, rms_disp, seed, backend="numpy", device="cuda"):
    """Returns (x, y, z) float32 arrays of n^3 particles in [0, box).

    backend "numpy" runs everything on the host; "torch" draws the same noise
    and transforms it on ``device``.
    """
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((n, n, n), dtype=np.float64)
    if backend == "torch":
        import torch

        t = torch.from_numpy(noise).to(device)
        del noise
        white = torch.fft.rfftn(t)
        del t
        kf = 2.0 * math.pi / box
        k1 = torch.fft.fftfreq(n, d=1.0 / n, device=device, dtype=torch.float64) * kf
        kz = torch.fft.rfftfreq(n, d=1.0 / n, device=device, dtype=torch.float64) * kf
        kx, ky, kzz = k1[:, None, None], k1[None, :, None], kz[None, None, :]
        k2 = kx * kx + ky * ky + kzz * kzz
        k2[0, 0, 0] = 1.0
        amp = torch.sqrt(torch.pow(k2, -0.5) * torch.exp(-4.0 * k2))
        amp[0, 0, 0] = 0.0
        delta_k = white * amp
        del white, amp
        psi = []
        for kc in (kx, ky, kzz):
            comp = torch.fft.irfftn(1j * (kc / k2) * delta_k, s=(n, n, n))
            psi.append(comp)
        del delta_k
        rms = torch.sqrt(sum((c * c).mean() for c in psi)).item()
        scale = rms_disp / rms
        q = (torch.arange(n, device=device, dtype=torch.float64) + 0.5) * (box / n)
        qs = (q[:, None, None], q[None, :, None], q[None, None, :])
        out = []
        for c, qa in zip(psi, qs):
            v = torch.remainder(qa + scale * c, box).to(torch.float32)
            v = torch.where(v >= box, torch.zeros_like(v), v)
            out.append(v.reshape(-1).cpu().numpy())
        return tuple(out)

    white = np.fft.rfftn(noise)
    del noise
    k1, kz = _kgrid(n, box, np)
    kx, ky, kzz = k1[:, None, None], k1[None, :, None], kz[None, None, :]
    k2 = kx * kx + ky * ky + kzz * kzz
    k2[0, 0, 0] = 1.0
    amp = np.sqrt(k2 ** -0.5 * np.exp(-4.0 * k2))
    amp[0, 0, 0] = 0.0
    delta_k = white * amp
    del white, amp
    psi = [np.fft.irfftn(1j * (kc / k2) * delta_k, s=(n, n, n), axes=(0, 1, 2))
           for kc in (kx, ky, kzz)]
    rms = math.sqrt(sum(float((c * c).mean()) for c in psi))
    scale = rms_disp / rms
    q = (np.arange(n, dtype=np.float64) + 0.5) * (box / n)
    qs = (q[:, None, None], q[None, :, None], q[None, None, :])
    out = []
    for c, qa in zip(psi, qs):
        v = np.remainder(qa + scale * c, box).astype(np.float32)
        v[v >= np.float32(box)] = 0.0
        out.append(np.ascontiguousarray(v.reshape(-1)))
    return tuple(out)


def workload_particles(name, backend="numpy", device="cuda"):
    w = WORKLOADS[name]
    return zeldovich(w["n"], w["box"], w["rms_disp"], w["seed"], backend, device)


def batch_boxes(n_boxes=64, seed=2000, n_lo=64, n_hi=256):
    """The batched workload's box list: particles per side log-uniform in
    [n_lo, n_hi], sides uniform in [200, 1000]; box b is seeded 2000 + b."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n_boxes):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        box = float(rng.uniform(200.0, 1000.0))
        out.append(dict(n=n, box=box, rms_disp=4.0, seed=2000 + b))
    return out


# A synthetic survey: a spherical footprint inside a padded box, less a
# stripe through it; data and randoms over it under a selection that falls
# along z; holes carved into the data (three inside, one cut by the edge).
SURVEY = dict(box=400.0, centre=(200.0, 200.0, 200.0), radius=140.0,
              stripe=((200.0, 260.0), 12.0),
              holes=((160.0, 160.0, 160.0, 26.0), (240.0, 160.0, 240.0, 22.0),
                     (150.0, 240.0, 220.0, 20.0), (200.0, 200.0, 325.0, 25.0)),
              kept_in_hole=0.03)


def _in_survey(p, s):
    c = np.asarray(s["centre"])
    inside = ((p - c) ** 2).sum(axis=1) <= s["radius"] ** 2
    (sx, sy), half = s["stripe"]
    stripe = (np.abs(p[:, 0] - sx) < half) & (np.abs(p[:, 1] - sy) < half)
    return inside & ~stripe


def survey(n_data, n_randoms, seed, selection=False, spec=SURVEY):
    """(data, randoms): each (x, y, z) float32 arrays inside the footprint,
    drawn uniformly (times a selection falling linearly from 1 at the bottom
    of the footprint to 0.4 at its top, when asked); the data thinned to
    ``kept_in_hole`` inside each hole."""
    rng = np.random.default_rng(seed)
    c = np.asarray(spec["centre"])
    R = spec["radius"]

    def draw(n, carve):
        out = np.empty((0, 3))
        while len(out) < n:
            p = c + (2.0 * rng.random((2 * n, 3)) - 1.0) * R
            p = p[_in_survey(p, spec)]
            if selection:
                keep = 1.0 - 0.6 * (p[:, 2] - (c[2] - R)) / (2.0 * R)
                p = p[rng.random(len(p)) <= keep]
            if carve:
                holes = np.zeros(len(p), bool)
                for hx, hy, hz, hr in spec["holes"]:
                    holes |= ((p - (hx, hy, hz)) ** 2).sum(axis=1) < hr * hr
                p = p[~holes | (rng.random(len(p)) <= spec["kept_in_hole"])]
            out = np.concatenate([out, p])
        out = out[:n].astype(np.float32)
        return out[:, 0].copy(), out[:, 1].copy(), out[:, 2].copy()

    return draw(n_data, True), draw(n_randoms, False)
