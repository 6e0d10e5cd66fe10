"""Seeded synthetic sphere ensembles for the five benchmark shapes.

No public dataset exists for this path; every workload is a seeded random
sequential addition (RSA) of sphere centres in a square at a fixed height,
with a minimum centre distance. numpy's PCG64 generator makes the positions
identical on every platform.

Shapes (all lengths in nm, vacuum wavelength in nm):

* ``c1``: 100 spheres r=100, n=1.52 at z=100 on glass (n=1.52) under air,
  l_max=m_max=3, TE from the top at normal incidence, 550 nm, linear lookup
  at 5 nm, GMRES tol 1e-8. The 2 um x 2 um square of the original shape
  needs 87% disk coverage at 210 nm minimum distance, above the ~55% RSA
  jamming limit, so the square is enlarged to 3 um x 3 um (38% coverage).
* ``c2``: 2000 spheres, same materials, 12 um square, TM at polar 30 deg
  (cos > 0: incidence from the glass side, the reference's convention),
  azimuth 0, cubic lookup at 5 nm.
* ``c3``: 5000 spheres r=80, n=2+0.01j at z=80 in a 20 um square, d_min=170,
  l_max=m_max=4, 600 nm, TE from the top, cubic lookup at 2 nm.
* ``c4``: the c3 geometry with 64 plane waves, polar angle pi - U[0, 45 deg]
  (from the top), azimuth U[0, 2 pi), TE/TM alternating.
* ``c5``: 10000 spheres r=100, n=1.52 at z=150 (mid-plane of a 300 nm film of
  n=1.8 between glass and air), 30 um square, d_min=210, l_max=m_max=3, 16
  plane waves at 550 nm (as c4), linear lookup at 5 nm.

``scaled(name, n)`` keeps a shape's density and optics with fewer spheres.
"""
import math

import numpy as np

SHAPES = {
    "c1": dict(n_spheres=100, side=3000.0, z=100.0, radius=100.0, n_particle=1.52, d_min=210.0, l_max=3,
               layers=([0, 0], [1.52, 1.0]), wavelength=550.0, resolution=5.0, kind="linear", tol=1e-8,
               waves=[(math.pi, 0.0, 0)]),
    "c2": dict(n_spheres=2000, side=12000.0, z=100.0, radius=100.0, n_particle=1.52, d_min=210.0, l_max=3,
               layers=([0, 0], [1.52, 1.0]), wavelength=550.0, resolution=5.0, kind="cubic", tol=1e-8,
               waves=[(math.pi / 6, 0.0, 1)]),
    "c3": dict(n_spheres=5000, side=20000.0, z=80.0, radius=80.0, n_particle=2.0 + 0.01j, d_min=170.0, l_max=4,
               layers=([0, 0], [1.52, 1.0]), wavelength=600.0, resolution=2.0, kind="cubic", tol=1e-6,
               waves=[(math.pi, 0.0, 0)]),
    "c4": dict(n_spheres=5000, side=20000.0, z=80.0, radius=80.0, n_particle=2.0 + 0.01j, d_min=170.0, l_max=4,
               layers=([0, 0], [1.52, 1.0]), wavelength=600.0, resolution=2.0, kind="cubic", tol=1e-6,
               waves=("random", 64)),
    "c5": dict(n_spheres=10000, side=30000.0, z=150.0, radius=100.0, n_particle=1.52, d_min=210.0, l_max=3,
               layers=([0, 300, 0], [1.52, 1.8, 1.0]), wavelength=550.0, resolution=5.0, kind="linear", tol=1e-6,
               waves=("random", 16)),
}


def rsa_positions(n, side, d_min, seed, max_batches=100000):
    """Random sequential addition of ``n`` centres in [0, side]^2.

    Candidates are drawn in batches; a cell grid with cell edge d_min/sqrt(2)
    holds at most one accepted centre per cell, so each test looks at the
    5 x 5 surrounding cells only.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cell = d_min / math.sqrt(2.0)
    nc = int(math.ceil(side / cell)) + 1
    grid = -np.ones((nc + 4, nc + 4), dtype=np.int64)
    pts = np.zeros((n, 2))
    count = 0
    d2 = d_min * d_min
    offs = np.array([(a, b) for a in range(-2, 3) for b in range(-2, 3)])
    for _ in range(max_batches):
        if count >= n:
            break
        cand = rng.uniform(0.0, side, size=(4096, 2))
        ci = (cand // cell).astype(np.int64) + 2
        nb = grid[ci[:, None, 0] + offs[None, :, 0], ci[:, None, 1] + offs[None, :, 1]]
        nbp = pts[np.maximum(nb, 0)]
        dd = ((nbp - cand[:, None, :]) ** 2).sum(-1)
        ok = ~np.any((nb >= 0) & (dd < d2), axis=1)
        for k in np.nonzero(ok)[0]:
            if count >= n:
                break
            cx, cy = ci[k]
            blk = grid[cx - 2:cx + 3, cy - 2:cy + 3]
            sel = blk[blk >= 0]
            if sel.size and np.any(((pts[sel] - cand[k]) ** 2).sum(-1) < d2):
                continue
            grid[cx, cy] = count
            pts[count] = cand[k]
            count += 1
    if count < n:
        raise RuntimeError("random sequential addition jammed at %d of %d centres" % (count, n))
    return pts


def plane_waves(spec, seed):
    """List of (polar, azimuth, polarization) for a shape's incident waves."""
    if spec[0] != "random":
        return list(spec)
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    r = spec[1]
    theta = rng.uniform(0.0, math.pi / 4, size=r)
    az = rng.uniform(0.0, 2 * math.pi, size=r)
    return [(math.pi - float(theta[i]), float(az[i]), i % 2) for i in range(r)]


def scaled(name, n_spheres):
    """Shape ``name`` with ``n_spheres`` centres at the same areal density."""
    s = dict(SHAPES[name])
    s["side"] = s["side"] * math.sqrt(n_spheres / s["n_spheres"])
    s["n_spheres"] = n_spheres
    return s


def build(name_or_spec, seed=0):
    """Return a dict with positions (N x 3), per-sphere data and the optics."""
    spec = dict(SHAPES[name_or_spec]) if isinstance(name_or_spec, str) else dict(name_or_spec)
    xy = rsa_positions(spec["n_spheres"], spec["side"], spec["d_min"], seed)
    pos = np.column_stack([xy, np.full(len(xy), spec["z"])])
    spec["positions"] = pos
    spec["plane_waves"] = plane_waves(spec["waves"], seed)
    return spec
