"""Seeded synthetic inputs for the benchmark and parity workloads.

Placement: random sequential addition of N unit spheres (a = 1) in a cubic
periodic box sized for volume fraction phi, L = (N (4 pi / 3) / phi)^(1/3);
a candidate whose minimum-image distance to any placed centre is below 2.0
is rejected.  Generalised forces are i.i.d. N(0, 1).  Everything is driven
by numpy's PCG64 with a fixed seed, so the GPU engine and the CPU oracle
see identical inputs.
"""
from __future__ import annotations

import math

import numpy as np


def box_length(n: int, phi: float, a: float = 1.0) -> float:
    return (n * (4.0 * math.pi / 3.0) * a ** 3 / phi) ** (1.0 / 3.0)


def rsa_positions(n: int, phi: float, seed: int = 42, dmin: float = 2.0,
                  max_tries: int = 2000000) -> tuple[np.ndarray, float]:
    """Random sequential addition in a periodic cube; returns (pos[n,3], L)."""
    L = box_length(n, phi)
    rng = np.random.default_rng(seed)
    ncell = max(1, int(L // dmin))
    cw = L / ncell
    cells: dict[tuple[int, int, int], list[int]] = {}
    pos = np.empty((n, 3))
    placed = 0
    tries = 0
    d2 = dmin * dmin
    while placed < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"RSA jammed after {placed} of {n} spheres (phi={phi})")
        p = rng.uniform(0.0, L, 3)
        c = tuple(int(v // cw) % ncell for v in p)
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    key = ((c[0] + dx) % ncell, (c[1] + dy) % ncell, (c[2] + dz) % ncell)
                    for q in cells.get(key, ()):
                        d = p - pos[q]
                        d -= L * np.round(d / L)
                        if d @ d < d2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            pos[placed] = p
            cells.setdefault(c, []).append(placed)
            placed += 1
    return pos, L


def forces(n_values: int, seed: int = 7, dtype=np.float64) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(n_values).astype(dtype)


# the workloads the library is measured on (F = 0, FT = 1, FTS = 2)
WORKLOADS = {
    "mob_f_n64_phi0.10_5shell": dict(version=0, n=64, phi=0.10, shells=5),
    "mob_fts_n1000_phi0.30": dict(version=2, n=1000, phi=0.30),
    "bd_f_n4096_phi0.20": dict(version=0, n=4096, phi=0.20),
    "mob_ft_n2048_phi0.25": dict(version=1, n=2048, phi=0.25),
}
