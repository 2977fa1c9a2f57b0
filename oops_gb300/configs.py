"""The synthetic workloads (seeded stand-ins for the configs the reference is
measured on; no public dataset is involved).  Each returns the bath, field,
pulse sequence and time grid of one CCE run."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .bath import diamond_bath


@dataclass
class Workload:
    name: str
    coords: np.ndarray      # Angstrom
    B: np.ndarray           # T
    cutoff: float           # Angstrom
    max_order: int          # CCE order (clusters of up to max_order spins)
    pulse_num: int          # CPMG pulses, 1 = Hahn
    nT: int
    t_max: float            # s

    @property
    def dt(self):
        return self.t_max / (self.nT - 1)


NV_AXIS = np.ones(3) / np.sqrt(3.0)


def tilted_field(mag, tilt_deg, azimuth):
    n = NV_AXIS
    e1 = np.array([1.0, -1.0, 0.0]) / np.sqrt(2.0)
    e2 = np.cross(n, e1)
    th = np.deg2rad(tilt_deg)
    d = np.cos(th) * n + np.sin(th) * (np.cos(azimuth) * e1 + np.sin(azimuth) * e2)
    return mag * d


def cce2_hahn(seed=2011):
    """CCE-2 Hahn echo: 2.0 nm sphere, 1.1 % 13C, B = 0.05 T along [111],
    cutoff 4.5 A, 201 points over [0, 2 ms]."""
    return Workload("cce2_hahn_r2.0nm_p1.1pct", diamond_bath(20.0, 0.011, seed),
                    0.05 * NV_AXIS, 4.5, 2, 1, 201, 2e-3)


def cce4_hahn(seed=4022):
    """CCE-4 Hahn echo: 3.0 nm sphere, 1.1 % 13C, B = 0.05 T along [111],
    cutoff 6 A, 401 points over [0, 4 ms]."""
    return Workload("cce4_hahn_r3.0nm_p1.1pct", diamond_bath(30.0, 0.011, seed),
                    0.05 * NV_AXIS, 6.0, 4, 1, 401, 4e-3)


def cce6_cpmg8(seed=6033):
    """CCE-6 CPMG-8: 4.0 nm sphere, 1.1 % 13C, |B| = 0.1 T tilted 3 degrees
    from [111] at a seeded azimuth, cutoff 7 A, 501 points over [0, 8 ms]."""
    rng = np.random.default_rng(seed + 1)
    B = tilted_field(0.1, 3.0, rng.uniform(0, 2 * np.pi))
    return Workload("cce6_cpmg8_r4.0nm_p1.1pct", diamond_bath(40.0, 0.011, seed),
                    B, 7.0, 6, 8, 501, 8e-3)


WORKLOADS = {"cce2": cce2_hahn, "cce4": cce4_hahn, "cce6": cce6_cpmg8}


def krylov_stress_cluster(k, seed=14016):
    """Large-cluster Krylov stress: k 13C spins drawn from the 1.1 % diamond
    lattice within 1.2 nm of a seeded centre (the nearest k occupied sites to
    it, so every k gets a cluster), B = 0.05 T along [111]."""
    rng = np.random.default_rng(seed)
    sites = diamond_bath(40.0, 0.011, seed)
    centre = sites[rng.integers(len(sites))]
    d = np.linalg.norm(sites - centre, axis=1)
    pick = np.argsort(d, kind="stable")[:k]
    return sites[pick], 0.05 * NV_AXIS
