"""Load golden fixtures and rebuild their inputs as oracle objects."""
import os

import numpy as np

import oracle.layers as olay
import oracle.physics as ophys
import oracle.special as osp

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def available(volume=False):
    """Fixture names: the radial-lookup solve cases, or (``volume=True``) the volume-lookup cases.
    (``pwe*`` fixtures hold plane-wave expansions only and are loaded by name.)"""
    names = sorted(f[:-4] for f in os.listdir(GOLDEN_DIR) if f.endswith(".npz") and not f.startswith("pwe"))
    return [n for n in names if n.startswith("vol") == volume]


def load(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))


def oracle_inputs(g):
    """(particles, layer_system, wavelength, kpar) for a fixture."""
    parts = [ophys.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                          m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    n_layers = [complex(x) if complex(x).imag else float(complex(x).real) for x in g["layer_n"]]
    ls = olay.LayerSystem([float(x) for x in g["thicknesses"]], n_layers)
    wl = float(g["wavelength"])
    return parts, ls, wl


def oracle_contour(g, ls, wl):
    wp = g["neff_waypoints"]
    return osp.sommerfeld_kpar_contour(wl, ls.refractive_indices,
                                       neff_waypoints=list(wp) if len(wp) else None,
                                       neff_resolution=float(g["neff_resolution"]))


def plane_wave(g, iw, cls=ophys.PlaneWave):
    polar, az, pol = g["waves"][iw]
    return cls(vacuum_wavelength=float(g["wavelength"]), polar_angle=float(polar), azimuthal_angle=float(az),
               polarization=int(pol), amplitude=1, reference_point=list(g["wave_reference_point"]))


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
