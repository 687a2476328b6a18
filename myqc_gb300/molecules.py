"""Seeded synthetic molecules for the benchmark workloads.

Water clusters: rigid monomers (O-H 0.9572 A, H-O-H 104.52 deg), O positions
uniform in a cube and rejection-sampled to O-O >= 2.7 A, orientations from a
uniform random unit quaternion, all drawn from numpy's PCG64 generator with a
recorded seed.  (H2O)_32 in a 9.5 A cube and (H2O)_64 in a 12 A cube are the
shapes of the precision and at-scale workloads.
"""
from __future__ import annotations

import numpy as np

from .formats import System, system_from_geometry

R_OH = 0.9572
ANGLE_HOH = 104.52


def water_monomer() -> np.ndarray:
    """O, H, H in Angstrom with O at the origin, molecule in the xy plane."""
    h = np.deg2rad(ANGLE_HOH) / 2
    return np.array([[0.0, 0.0, 0.0], [R_OH * np.sin(h), R_OH * np.cos(h), 0.0],
                     [-R_OH * np.sin(h), R_OH * np.cos(h), 0.0]])


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(nmol: int, box: float, seed: int = 0, min_oo: float = 2.7, max_tries: int = 100000):
    """(symbols, xyz in Angstrom) of a seeded (H2O)_nmol cluster."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centers = []
    tries = 0
    while len(centers) < nmol:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place the waters; enlarge the box")
        c = rng.uniform(0.0, box, size=3)
        if all(np.linalg.norm(c - o) >= min_oo for o in centers):
            centers.append(c)
    mono = water_monomer()
    sym, xyz = [], []
    for c in centers:
        R = random_rotation(rng)
        for s, r in zip("OHH", mono):
            sym.append(s)
            xyz.append(c + R @ r)
    return sym, np.array(xyz)


def water_cluster_system(nmol: int, box: float, seed: int = 0, calc_mp2: bool = True) -> System:
    sym, xyz = water_cluster(nmol, box, seed)
    return system_from_geometry(sym, xyz, calc_mp2=calc_mp2)
