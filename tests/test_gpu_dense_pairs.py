"""The thread-per-pair split-precision dense builder (k_matrix_pairs: FP32
terms at a split of its own, lattice images enumerated per pair, half-space
reciprocal table; FTS with the reference split's G term) against the FP64
builder at the reference's split (src/ewald.c:1092-1677): largest entry
error <= 1e-6 of the largest entry, on the dense workload itself (FTS,
N = 1000, phi 0.30), on a rectangular box, and on a box whose cutoff spans
several lattice images; the kernel that ran is checked by name."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _mats(lib, version, pos, box):
    from libstokes_gb300 import FP64, MIXED, System, abi
    a = System(version, pos, box)
    a.set_precision(FP64)
    b = System(version, pos, box)
    b.set_precision(MIXED)
    m64 = a.matrix()
    lib.stokes_gpu_kprof_begin(b.sp, 16)
    m32 = b.matrix()
    names = abi.kernel_profile(lib, b.sp)
    return a, b, m64, m32, names


@pytest.mark.parametrize("version,n,phi", [(2, 1000, 0.30), (0, 300, 0.1), (1, 64, 0.02)])
def test_pair_builder_against_fp64(lib, version, n, phi):
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=42)
    a, b, m64, m32, names = _mats(lib, version, pos, (L, L, L))
    assert "k_matrix_pairs" in names, names
    err = np.abs(m32 - m64).max() / np.abs(m64).max()
    assert 0.0 < err < 1e-6, err
    # the matrix route of the product (atimes_3all_matrix; FTS applies the
    # extracted form's transform) against the FP64 product at the mixed bar
    x = np.random.default_rng(3).standard_normal(m64.shape[0])
    assert rel_l2(b.atimes_matrix(x), a.atimes(x)) < 1e-6
    a.close()
    b.close()


def test_pair_builder_rectangular_box(lib):
    rng = np.random.default_rng(11)
    box = (14.0, 18.0, 11.0)
    n = 90
    pos = np.zeros((n, 3))
    for i in range(n):                      # rejection: centres 2 apart
        while True:
            p = rng.uniform(0, 1, 3) * box
            d = pos[:i] - p
            d -= np.array(box) * np.rint(d / np.array(box))
            if i == 0 or np.min(np.linalg.norm(d, axis=1)) > 2.05:
                pos[i] = p
                break
    # unwrapped coordinates: the builder takes the minimum image itself
    shifted = pos.copy()
    shifted[::3] += np.array(box) * np.array([1.0, -2.0, 3.0])
    from libstokes_gb300 import MIXED, System
    for version in (1, 2):
        a, b, m64, m32, names = _mats(lib, version, pos, box)
        assert "k_matrix_pairs" in names, names
        err = np.abs(m32 - m64).max() / np.abs(m64).max()
        assert 0.0 < err < 1e-6, (version, err)
        c = System(version, shifted, box)
        c.set_precision(MIXED)
        ms = c.matrix()
        assert np.abs(ms - m64).max() / np.abs(m64).max() < 1e-6, version
        for s in (a, b, c):
            s.close()
