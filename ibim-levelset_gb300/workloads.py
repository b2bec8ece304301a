"""Solve workloads of the benchmark and the parity tests (seeded synthetic molecules).

Each workload is a molecule plus the input.cfg values of the reference's path
(data/input.cfg keys; geometry explicit, lengths in Angstrom):
  born        one ion, R = 2 A, q = +1, 64^3 grid over [-6, 6)^3, p = 4, leaf <= 64, kappa = 0,
              eps 1/80, GMRES(30) to 1e-6 (the Born ion of the benchmark's first configuration)
  protein2000 synthetic protein of 2,000 atoms (seed 1,000,000), h = 0.5 A, p = 5, kappa = 0.125,
              eps 2/80, reinit 20 steps (the benchmark's second configuration)
  protein20k  20,000 atoms (seed 2,000,000), h = 0.25 A, p = 6 (third configuration)
Values the configurations leave open are fixed here: tube thickness 3 (Born) / 2 (reference
default, data/input.cfg), fmm_maxpoint 64 (Born) / 128, fmm_maxlevel 10, tau 1, GMRES(30),
tolerance 1e-6, at most 200 iterations.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

import synth


@dataclass
class Workload:
    name: str
    mol: synth.Molecule
    geo: synth.Geometry
    thickness: int
    np_: int
    maxpoint: int
    kappa: float
    dI: float
    dE: float
    reinit_steps: int = 20
    tol: float = 1e-6
    restart: int = 30
    maxiter: int = 200
    maxlevel: int = 10
    tau: float = 1.0
    thres: float = 1e-4

    @property
    def reinit_t(self) -> float:
        return synth.reinit_time(self.reinit_steps, self.geo.h)

    @property
    def init(self) -> float:
        return -2.0 * max(self.geo.n)

    def config(self, precision: int = 0):
        import ibim

        return ibim.default_config(lo=self.geo.lo, h=self.geo.h, n=self.geo.n, band=8, init=self.init, probe=1.4,
                                   reinit_t=self.reinit_t, thickness=self.thickness, thres=self.thres, np=self.np_,
                                   maxpoint=self.maxpoint, maxlevel=self.maxlevel, kappa=self.kappa, dE=self.dE,
                                   dI=self.dI, tau=self.tau, restart=self.restart, maxiter=self.maxiter,
                                   tol=self.tol, precision=precision)

    def describe(self) -> dict:
        return dict(workload=self.name, atoms=self.mol.n, grid=list(self.geo.n), h=self.geo.h,
                    chebyshev_order=self.np_, leaf_max_points=self.maxpoint, tube_thickness=self.thickness,
                    kappa=self.kappa, eps_in=self.dI, eps_out=self.dE, reinit_steps=self.reinit_steps,
                    gmres_restart=self.restart, gmres_tol=self.tol)


def born() -> Workload:
    return Workload("born_ion_64cubed", synth.born_ion(), synth.born_geometry(), thickness=3, np_=4, maxpoint=64,
                    kappa=0.0, dI=1.0, dE=80.0)


def protein(n_atoms: int = 2000, seed: int = 1_000_000, h: float = 0.5, order: int = 5, maxpoint: int = 128,
            kappa: float = 0.125) -> Workload:
    mol = synth.synthetic_protein(n_atoms, seed)
    return Workload(f"synthetic_protein_{n_atoms}_atoms_h{h}", mol, synth.padded_geometry(mol, h), thickness=2,
                    np_=order, maxpoint=maxpoint, kappa=kappa, dI=2.0, dE=80.0)


def protein2000() -> Workload:
    return protein(2000, 1_000_000, 0.5, 5)


def protein20k() -> Workload:
    return protein(20000, 2_000_000, 0.25, 6)


def born_energy(q: float = 1.0, R: float = 2.0, eps_in: float = 1.0, eps_out: float = 80.0) -> float:
    """Analytic Born solvation energy -(q^2 / 8 pi R)(1/eps_in - 1/eps_out), e^2/A."""
    return -(q * q / (8.0 * np.pi * R)) * (1.0 / eps_in - 1.0 / eps_out)
