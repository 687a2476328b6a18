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


# Standard geometries of the batched workload's small molecules, Angstrom.
# Bond lengths and angles are the experimental equilibrium values tabulated in
# the NIST Computational Chemistry Comparison and Benchmark Database (CCCBDB,
# NIST Standard Reference Database 101, "experimental geometries"):
#   H2 r 0.741; HF r 0.917; H2O r 0.9572, 104.52 deg; NH3 r 1.012, HNH 106.67
#   deg; CH4 r 1.087 (Td); CO r 1.128; CO2 r 1.160 (linear); C2H2 r(CC) 1.203,
#   r(CH) 1.063 (linear); HCN r(CH) 1.065, r(CN) 1.153 (linear).
def _nh3():
    r, a = 1.012, np.deg2rad(106.67)
    # N on the z axis above the plane of the three H: in-plane radius rho from
    # the H-H distance d, height h from r
    d = 2 * r * np.sin(a / 2)
    rho = d / np.sqrt(3.0)
    h = np.sqrt(r * r - rho * rho)
    H = [[rho * np.cos(t), rho * np.sin(t), 0.0] for t in (0.0, 2 * np.pi / 3, 4 * np.pi / 3)]
    return ["N", "H", "H", "H"], np.array([[0.0, 0.0, h]] + H)


def _ch4():
    r = 1.087 / np.sqrt(3.0)
    H = [[r, r, r], [-r, -r, r], [-r, r, -r], [r, -r, -r]]
    return ["C", "H", "H", "H", "H"], np.array([[0.0, 0.0, 0.0]] + H)


STANDARD_GEOMETRIES = {
    "H2": (["H", "H"], np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.741]])),
    "HF": (["F", "H"], np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.917]])),
    "H2O": (["O", "H", "H"], water_monomer()),
    "NH3": _nh3(),
    "CH4": _ch4(),
    "CO": (["C", "O"], np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.128]])),
    "CO2": (["C", "O", "O"], np.array([[0.0, 0.0, 0.0], [0.0, 0.0, -1.160], [0.0, 0.0, 1.160]])),
    "C2H2": (["C", "C", "H", "H"], np.array([[0.0, 0.0, -0.6015], [0.0, 0.0, 0.6015], [0.0, 0.0, -1.6645],
                                              [0.0, 0.0, 1.6645]])),
    "HCN": (["H", "C", "N"], np.array([[0.0, 0.0, -1.065], [0.0, 0.0, 0.0], [0.0, 0.0, 1.153]])),
}
BATCH_KINDS = list(STANDARD_GEOMETRIES) + [f"(H2O){k}" for k in range(2, 9)]


def standard_geometry(kind: str):
    """(symbols, xyz) of one batch kind; (H2O)_k clusters are the seeded cluster
    generator's geometry with seed k in a cube of side (27 k)^(1/3) + 1 A."""
    if kind in STANDARD_GEOMETRIES:
        sym, xyz = STANDARD_GEOMETRIES[kind]
        return list(sym), np.array(xyz, dtype=float)
    k = int(kind[5:])
    return water_cluster(k, (27.0 * k) ** (1 / 3) + 1.0, k)


def batch_workload(count: int, seed: int = 0, sigma: float = 0.05):
    """`count` closed-shell molecules drawn uniformly from BATCH_KINDS, every
    Cartesian coordinate perturbed by N(0, sigma A); returns (kinds, Systems)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kinds, systems = [], []
    for _ in range(count):
        kind = BATCH_KINDS[int(rng.integers(len(BATCH_KINDS)))]
        sym, xyz = standard_geometry(kind)
        xyz = xyz + rng.normal(0.0, sigma, size=xyz.shape)
        kinds.append(kind)
        systems.append(system_from_geometry(sym, xyz, calc_mp2=False))
    return kinds, systems
