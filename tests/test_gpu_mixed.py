"""Mixed-precision product against the FP64 path on the same inputs.

Bar: relative L2 error <= 1e-6 (the mixed-path tolerance).  The FP64 path is
itself pinned to the reference at 1e-12 (test_gpu_products.py)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-6


def _pair(version, n, phi, seed=1, shear=(0, 0.0)):
    from libstokes_gb300 import FP64, MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=seed)
    x = np.random.default_rng(seed + 100).standard_normal((3, 6, 11)[version] * n)
    a = System(version, pos, (L, L, L))
    b = System(version, pos, (L, L, L))
    for s in (a, b):
        s.set_misc(0.0, *shear)
    a.set_precision(FP64)
    b.set_precision(MIXED)
    return a, b, x


@pytest.mark.parametrize("version,n,phi", [(0, 200, 0.2), (1, 300, 0.25), (2, 200, 0.3),
                                           (2, 1000, 0.3), (0, 1500, 0.2)])
def test_mixed_accuracy(lib, version, n, phi):
    a, b, x = _pair(version, n, phi)
    y64 = a.atimes(x)
    ymx = b.atimes(x)
    err = rel_l2(ymx, y64)
    assert err < TOL, err
    a.close()
    b.close()


@pytest.mark.parametrize("version,mode,shift", [(0, 1, 3.1), (2, 2, -4.4), (1, 1, 0.0)])
def test_mixed_shear(lib, version, mode, shift):
    a, b, x = _pair(version, 300, 0.2, seed=4, shear=(mode, shift))
    err = rel_l2(b.atimes(x), a.atimes(x))
    assert err < TOL, err
    a.close()
    b.close()


def test_mixed_unwrapped_positions(lib):
    """Positions outside the primary cell give the same product."""
    from libstokes_gb300 import MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(150, 0.2, seed=8)
    x = np.random.default_rng(9).standard_normal(3 * 150)
    shifted = pos + L * np.random.default_rng(10).integers(-3, 4, pos.shape)
    s1 = System(0, pos, (L, L, L))
    s2 = System(0, shifted, (L, L, L))
    s1.set_precision(MIXED)
    s2.set_precision(MIXED)
    assert rel_l2(s2.atimes(x), s1.atimes(x)) < 1e-6
    s1.close()
    s2.close()


def test_mixed_rejects_unsupported(lib):
    from libstokes_gb300 import MIXED, GPUError, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(20, 0.2, seed=2)
    s = System(0, pos, (L, L, L))
    s.set_radius(np.ones(20))
    s.set_precision(MIXED)
    with pytest.raises(GPUError):
        s.atimes(np.ones(60))
    s.close()
