"""Synthetic 13C baths on the diamond lattice (the configs' seeded inputs).

Diamond: lattice constant a (Angstrom), fcc lattice with the two-atom basis
(0,0,0) and (1/4,1/4,1/4)a.  The NV sits at the origin: the vacancy site
(origin) and the nitrogen site -(a/4)(1,1,1) hold no 13C.  Every other site
within `radius` (Angstrom) of the origin is 13C with probability `abundance`,
drawn with numpy's PCG64 generator from `seed` (identical on every platform).
The reference reads baths from .xyz files (cSpinSourceFromFile,
src/source/spin/SpinCollection/SpinSource.cpp:55-79) or draws uniform random
positions (cSpinSourceUniformRandom :112-129); a lattice generator is new.
"""
from __future__ import annotations

import numpy as np

DIAMOND_A = 3.567


def diamond_sites(radius, a=DIAMOND_A):
    n = int(np.ceil(radius / a)) + 1
    r = np.arange(-n, n + 1)
    cells = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    fcc = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    basis = np.concatenate([fcc, fcc + 0.25])
    pts = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    d = np.linalg.norm(pts, axis=1)
    keep = d <= radius
    pts, d = pts[keep], d[keep]
    nsite = -(a / 4.0) * np.ones(3)
    far = (d > 1e-6) & (np.linalg.norm(pts - nsite, axis=1) > 1e-6)
    pts, d = pts[far], d[far]
    # deterministic order: by distance, then lexicographic
    o = np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0], np.round(d, 9)))
    return pts[o]


def diamond_bath(radius, abundance, seed, a=DIAMOND_A):
    sites = diamond_sites(radius, a)
    rng = np.random.default_rng(seed)
    occ = rng.random(sites.shape[0]) < abundance
    return sites[occ].copy()


def read_xyz(path):
    """cSpinSourceFromFile format: count, then 'isotope x y z' lines."""
    with open(path) as f:
        n = int(f.readline().split()[0])
        rows = [f.readline().split() for _ in range(n)]
    return np.array([[float(x) for x in r[1:4]] for r in rows]), [r[0] for r in rows]
