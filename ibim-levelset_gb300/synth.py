"""Seeded synthetic molecules and solve geometries for the IBIM Poisson-Boltzmann path.

The reference (ibim-levelset) reads real proteins from PQR files (molecule.h:21-50:
lines starting with ``ATOM``, whitespace tokens 5..9 = x y z charge radius).  The
workloads here are synthetic proteins written in the same format so that the
reference's own loader reads them unchanged.

Generator (fixed here, deterministic on every machine):
  * PRNG: SplitMix64 (Steele, Lea & Flood 2014), uniform doubles from the top 53 bits,
    normals by Box-Muller.  Seed = config index * 10**6 + molecule index.
  * Backbone: half of the atoms (rounded up).  A self-avoiding walk from the origin with
    3.8 A steps in isotropic random directions; a step is rejected when it lands within
    3.0 A of an earlier backbone centre or leaves the confinement sphere of radius
    2.2 * n_atoms**(1/3) A.  After 64 rejected tries the walk backtracks one atom.
  * Side atoms: the other half, each uniform in the 2 A ball around a random backbone atom.
  * Radii uniform in [1.2, 2.0] A; charges N(0, 0.4^2) e, shifted by (round(sum) - sum)/n
    per atom so that the net charge is an integer.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_MASK = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 generator (public-domain algorithm by Steele, Lea and Flood)."""

    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def normal(self) -> float:
        u1 = self.uniform()
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(1.0 - u1)) * math.cos(2.0 * math.pi * u2)

    def direction(self):
        z = 2.0 * self.uniform() - 1.0
        phi = 2.0 * math.pi * self.uniform()
        s = math.sqrt(max(0.0, 1.0 - z * z))
        return (s * math.cos(phi), s * math.sin(phi), z)


@dataclass
class Molecule:
    """Atoms of one molecule: centres (n,3) [A], charges (n,) [e], radii (n,) [A]."""

    centers: np.ndarray
    charges: np.ndarray
    radii: np.ndarray

    @property
    def n(self) -> int:
        return int(self.centers.shape[0])

    def to_pqr(self, path: str) -> None:
        with open(path, "w") as f:
            for i in range(self.n):
                x, y, z = self.centers[i]
                f.write(f"ATOM  {i + 1:5d}  C   SYN {i // 8 + 1:5d}    {x:.10f} {y:.10f} {z:.10f} "
                        f"{self.charges[i]:.12f} {self.radii[i]:.12f}\n")

    @staticmethod
    def from_pqr(path: str) -> "Molecule":
        """Read ``ATOM`` lines as molecule.h:21-50 does (tokens 5..9 = x y z q r)."""
        c, q, r = [], [], []
        with open(path) as f:
            for line in f:
                if line.startswith("ATOM"):
                    t = line.split()
                    c.append((float(t[5]), float(t[6]), float(t[7])))
                    q.append(float(t[8]))
                    r.append(float(t[9]))
        return Molecule(np.asarray(c, dtype=np.float64).reshape(-1, 3), np.asarray(q, dtype=np.float64),
                        np.asarray(r, dtype=np.float64))


def born_ion() -> Molecule:
    """One atom at the origin, radius 2.0 A, charge +1 e."""
    return Molecule(np.zeros((1, 3)), np.ones(1), np.full(1, 2.0))


def synthetic_protein(n_atoms: int, seed: int) -> Molecule:
    """Synthetic protein of ``n_atoms`` atoms (see the module docstring)."""
    if n_atoms < 1:
        raise ValueError("n_atoms must be >= 1")
    rng = SplitMix64(seed)
    n_bb = (n_atoms + 1) // 2
    n_side = n_atoms - n_bb
    r_conf = 2.2 * n_atoms ** (1.0 / 3.0)
    cell = 3.0
    buckets: dict = {}

    def key(p):
        return (math.floor(p[0] / cell), math.floor(p[1] / cell), math.floor(p[2] / cell))

    def clash(p):
        kx, ky, kz = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for q in buckets.get((kx + dx, ky + dy, kz + dz), ()):
                        if (p[0] - q[0]) ** 2 + (p[1] - q[1]) ** 2 + (p[2] - q[2]) ** 2 < 9.0:
                            return True
        return False

    bb = [(0.0, 0.0, 0.0)]
    buckets.setdefault(key(bb[0]), []).append(bb[0])
    budget = 1000 * n_bb + 10000
    while len(bb) < n_bb:
        budget -= 1
        if budget < 0:
            raise RuntimeError("backbone walk did not finish")
        last = bb[-1]
        placed = False
        for _ in range(64):
            d = rng.direction()
            p = (last[0] + 3.8 * d[0], last[1] + 3.8 * d[1], last[2] + 3.8 * d[2])
            if p[0] * p[0] + p[1] * p[1] + p[2] * p[2] > r_conf * r_conf:
                continue
            if clash(p):
                continue
            bb.append(p)
            buckets.setdefault(key(p), []).append(p)
            placed = True
            break
        if not placed and len(bb) > 1:
            q = bb.pop()
            buckets[key(q)].remove(q)
    centers = list(bb)
    for _ in range(n_side):
        j = min(int(rng.uniform() * n_bb), n_bb - 1)
        d = rng.direction()
        rad = 2.0 * rng.uniform() ** (1.0 / 3.0)
        b = bb[j]
        centers.append((b[0] + rad * d[0], b[1] + rad * d[1], b[2] + rad * d[2]))
    radii = np.array([1.2 + 0.8 * rng.uniform() for _ in range(n_atoms)])
    q = np.array([0.4 * rng.normal() for _ in range(n_atoms)])
    q += (round(float(q.sum())) - float(q.sum())) / n_atoms
    return Molecule(np.asarray(centers, dtype=np.float64), q, radii)


@dataclass
class Geometry:
    """Uniform grid: origin ``lo`` (3,), spacing ``h``, sizes ``n`` (3,) (levelset.h:33-48)."""

    lo: tuple
    h: float
    n: tuple

    @property
    def cells(self) -> int:
        return int(self.n[0]) * int(self.n[1]) * int(self.n[2])


def padded_geometry(mol: Molecule, h: float, probe: float = 1.4, band: int = 8, extra: float = 2.0) -> Geometry:
    """Bounding box of (c +- (R + probe)) padded by band*h + extra A, spacing h.

    The padding keeps every cell that levelset::expand touches (levelset.cpp:91-109:
    +-((R+probe)/h + band) cells around each centre) inside the grid.
    """
    lo = (mol.centers - (mol.radii + probe)[:, None]).min(axis=0) - (band * h + extra)
    hi = (mol.centers + (mol.radii + probe)[:, None]).max(axis=0) + (band * h + extra)
    n = tuple(int(math.ceil((hi[a] - lo[a]) / h)) + 1 for a in range(3))
    return Geometry(tuple(float(v) for v in lo), float(h), n)


def born_geometry() -> Geometry:
    """64^3 grid over the cube padded 4 A around the Born ion's sphere: [-6, 6)^3, h = 0.1875 A."""
    return Geometry((-6.0, -6.0, -6.0), 0.1875, (64, 64, 64))


def reinit_time(steps: int, h: float, cfl: float = 0.5) -> float:
    """Pseudo-time that makes levelset::reinitialize take exactly ``steps`` steps.

    levelset.cpp:192-195 takes floor(T / (cfl*h)) + 1 steps; T = (steps - 1/2) * cfl * h.
    """
    return (steps - 0.5) * cfl * h
