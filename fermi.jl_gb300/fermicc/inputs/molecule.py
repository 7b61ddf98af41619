"""Molecules for the coupled-cluster workloads: one water and seeded water clusters.

Fermi.jl builds a ``Molecule`` from an xyz string (src/Core/Molecule.jl:60-73);
this module produces the same information (element symbols and Cartesian
positions, Angstrom) for the workloads the coupled-cluster path is measured on.

Water-cluster generator (the seeded synthetic stand-in for a dataset of
geometries): oxygen atoms sit on an nx x ny x nz cubic lattice with 2.85 A
spacing; every oxygen coordinate is jittered by N(0, 0.1 A); each molecule is a
rigid water (O-H 0.9572 A, H-O-H 104.52 deg) rotated by a uniformly random
(Haar) rotation drawn from a unit quaternion.  Everything is drawn from one
``numpy.random.Generator(PCG64(seed))`` so a (lattice, seed) pair names one
geometry on every machine.
"""
from __future__ import annotations

import numpy as np

# Water at the geometry printed in Fermi's README (Angstrom): O, H, H.
README_WATER = [
    ("O", np.array([1.2091536548, 1.7664118189, -0.0171613972])),
    ("H", np.array([2.1984800075, 1.7977100627, 0.0121161719])),
    ("H", np.array([0.9197881882, 2.4580185570, 0.6297938830])),
]

R_OH = 0.9572
THETA_HOH = np.deg2rad(104.52)
SPACING = 2.85
JITTER = 0.1


def _rigid_water_body() -> np.ndarray:
    """H positions relative to O in the body frame (rows: H1, H2)."""
    half = THETA_HOH / 2
    return np.array([[R_OH * np.sin(half), 0.0, R_OH * np.cos(half)],
                     [-R_OH * np.sin(half), 0.0, R_OH * np.cos(half)]])


def _quat_to_rot(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def water_cluster(lattice: tuple[int, int, int], seed: int) -> list[tuple[str, np.ndarray]]:
    rng = np.random.Generator(np.random.PCG64(seed))
    nx, ny, nz = lattice
    body = _rigid_water_body()
    atoms = []
    for ix in range(nx):
        for iy in range(ny):
            for iz in range(nz):
                o = SPACING * np.array([ix, iy, iz], dtype=np.float64) + rng.normal(0.0, JITTER, 3)
                q = rng.normal(size=4)
                q /= np.linalg.norm(q)
                R = _quat_to_rot(q)
                atoms.append(("O", o))
                for h in body:
                    atoms.append(("H", o + R @ h))
    return atoms


LATTICES = {4: (2, 2, 1), 6: (2, 3, 1), 8: (2, 2, 2), 12: (3, 2, 2)}


def waters(n: int, seed: int) -> list[tuple[str, np.ndarray]]:
    """(H2O)n on its lattice: 4 -> 2x2x1, 6 -> 2x3x1, 8 -> 2x2x2, 12 -> 3x2x2.

    n = 1 returns the README water; n = 2 a 2x1x1 dimer (small test case)."""
    if n == 1:
        return [(e, p.copy()) for e, p in README_WATER]
    if n == 2:
        return water_cluster((2, 1, 1), seed)
    return water_cluster(LATTICES[n], seed)


def to_xyz(atoms) -> str:
    return "\n".join(f"{e} {p[0]:.10f} {p[1]:.10f} {p[2]:.10f}" for e, p in atoms)
