"""GPU parity at the measured workloads' own sizes, against the CPU oracle
(the C restatement of src/ewald.c:519-1081, pinned to the reference's
outputs by test_oracle_golden.py).

  * FTS, N = 1000, phi 0.30 (the headline product): the whole product,
    FP64 path at 1e-12 and mixed path at 1e-6 relative L2;
  * FT, N = 2048, phi 0.25 and F, N = 4096, phi 0.20: sampled output rows
    (three slices of particles spread over the system), FP64 at 1e-12 and
    mixed at 1e-6 relative L2 over the sampled rows.

Inputs are the seeded placements and forces the benchmark uses
(libstokes_gb300.workloads); the split is libstokes' default (xi =
sqrt(pi)/L, eps 1e-12) for the struct, from which the GPU path takes its
own tuned FP64 split or mixed split."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL64 = 1e-12
TOLMIX = 1e-6


def _oracle(version, pos, L):
    from oracle.oracle import Oracle
    o = Oracle(version, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    o.set_threads(os.cpu_count() or 1)
    return o


def _rows(y, c, slices):
    return np.concatenate([y[c * i0:c * i1] for i0, i1 in slices])


def test_headline_fts_n1000_full_product(lib):
    from libstokes_gb300 import System, abi
    from libstokes_gb300.workloads import forces, rsa_positions
    pos, L = rsa_positions(1000, 0.30, seed=42)
    x = forces(11 * 1000, seed=7)
    yo = _oracle(2, pos, L).atimes(x)
    s = System(2, pos, (L, L, L))
    y64 = s.atimes(x)
    e64 = rel_l2(y64, yo)
    s.set_precision(abi.MIXED)
    ymx = s.atimes(x)
    emx = rel_l2(ymx, yo)
    s.close()
    assert e64 < TOL64, e64
    assert emx < TOLMIX, emx


@pytest.mark.parametrize("version,n,phi", [(1, 2048, 0.25), (0, 4096, 0.20)])
def test_large_configs_sampled_rows(lib, version, n, phi):
    from libstokes_gb300 import System, abi
    from libstokes_gb300.workloads import forces, rsa_positions
    c = (3, 6, 11)[version]
    pos, L = rsa_positions(n, phi, seed=42)
    x = forces(c * n, seed=7)
    o = _oracle(version, pos, L)
    slices = [(0, 24), (n // 2 - 12, n // 2 + 12), (n - 24, n)]
    yo = np.zeros(c * n)
    for i0, i1 in slices:
        yo += o.atimes_rows(x, i0, i1)
    ref = _rows(yo, c, slices)
    s = System(version, pos, (L, L, L))
    y64 = _rows(s.atimes(x), c, slices)
    s.set_precision(abi.MIXED)
    ymx = _rows(s.atimes(x), c, slices)
    s.close()
    assert rel_l2(y64, ref) < TOL64, rel_l2(y64, ref)
    assert rel_l2(ymx, ref) < TOLMIX, rel_l2(ymx, ref)
