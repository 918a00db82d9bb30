"""GPU parity of the free-space (non-periodic) operator: atimes_nonewald_3all,
make_matrix_mob_nonewald_3all, atimes_nonewald_3all_matrix and the
dispatchers atimes_3all / make_matrix_mob_3all / atimes_3all_matrix on an
open system (sys->periodic == 0), against the reference's own outputs
(tests/golden/nonewald.npz) and the CPU oracle.

Tolerance: 1e-12 relative L2 (the FP64 bar); dense matrices 1e-12 of the
largest entry."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_open_oracle, make_open_system, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _mat_err(m, ref):
    return np.abs(m - ref).max() / np.abs(ref).max()


def test_products_golden(lib, nonewald):
    for name, case in nonewald.items():
        if "x" not in case:
            continue
        s = make_open_system(case)
        for f in (s.atimes_nonewald, s.atimes_3all):
            y = f(case["x"])
            assert rel_l2(y, case["y"]) < TOL, (name, f.__name__, rel_l2(y, case["y"]))
        s.close()


def test_matrices_golden(lib, nonewald):
    for name, case in nonewald.items():
        if "mat" not in case:
            continue
        s = make_open_system(case)
        assert _mat_err(s.matrix_nonewald(), case["mat"]) < TOL, name
        assert _mat_err(s.matrix_3all(), case["mat"]) < TOL, name
        if "x" in case:
            for f in (s.atimes_nonewald_matrix, s.atimes_3all_matrix):
                y = f(case["x"])
                assert rel_l2(y, case["y"]) < TOL, (name, f.__name__)
        s.close()


def test_nonewald_on_a_periodic_system(lib, nonewald):
    """atimes_nonewald_3all ignores sys->periodic (src/non-ewald.c:330): on a
    periodic system it still gives the free-space product, and the Ewald
    product of the same system is unchanged afterwards."""
    case = nonewald["r12_v2_poly"]
    s = make_open_system(case, periodic=True)
    y_ewald = s.atimes(case["x"])
    assert rel_l2(s.atimes_nonewald(case["x"]), case["y"]) < TOL
    assert _mat_err(s.matrix_nonewald(), case["mat"]) < TOL
    assert rel_l2(s.atimes(case["x"]), y_ewald) < 1e-15
    assert rel_l2(y_ewald, case["y"]) > 1e-3      # a different operator
    s.close()


def test_lattice_entry_points_refuse_open_systems(lib, nonewald):
    from libstokes_gb300 import abi
    case = nonewald["r12_v0_mono"]
    s = make_open_system(case)
    y = np.zeros(s.n)
    lib.atimes_ewald_3all(s.n, abi._d(case["x"]), abi._d(y), C.cast(s.sp, C.c_void_p))
    assert lib.stokes_gpu_last_error() == abi.STOKES_GPU_ENOTPERIODIC
    assert np.isnan(y).all()
    # the status-returning form dispatches like atimes_3all
    y = np.zeros(s.n)
    assert lib.stokes_gpu_atimes(s.sp, abi._d(case["x"]), abi._d(y)) == 0
    assert rel_l2(y, case["y"]) < TOL
    s.close()


def test_mixed_mode_product(lib, nonewald):
    """Mixed precision on an open system: FP32 pair terms with compensated
    sums (open_f32.cu) against the reference's products at the mixed bar
    (1e-6 relative L2); the dense matrix stays FP64."""
    from libstokes_gb300 import abi
    for name, case in nonewald.items():
        if "x" not in case:
            continue
        s = make_open_system(case)
        s.set_precision(abi.MIXED)
        err = rel_l2(s.atimes_3all(case["x"]), case["y"])
        assert err < 1e-6, (name, err)
        if "mat" in case:
            assert _mat_err(s.matrix_3all(), case["mat"]) < TOL
        s.close()


@pytest.mark.parametrize("version", [0, 1, 2])
def test_mixed_mode_large(lib, version):
    """N = 4000 polydisperse spheres with slip: mixed against FP64."""
    from libstokes_gb300 import abi
    from libstokes_gb300.workloads import rsa_positions
    rng = np.random.default_rng(31 + version)
    pos, _ = rsa_positions(4000, 0.25, seed=7 + version)
    case = dict(meta=np.array([version, 1.0]), pos=pos, a=rng.uniform(0.8, 1.2, 4000),
                slip=rng.uniform(0.0, 0.5, 4000))
    s = make_open_system(case)
    x = rng.standard_normal(s.n)
    y64 = s.atimes_3all(x)
    s.set_precision(abi.MIXED)
    assert rel_l2(s.atimes_3all(x), y64) < 1e-6
    s.close()


@pytest.mark.parametrize("version", [0, 1, 2])
def test_against_oracle_large(lib, version):
    """N = 1500 polydisperse spheres with the rmin clamp active for close
    pairs: every pair of the O(N^2) sum against the oracle."""
    from libstokes_gb300.workloads import rsa_positions
    rng = np.random.default_rng(17 + version)
    pos, _ = rsa_positions(1500, 0.2, seed=3 + version)
    case = dict(meta=np.array([version, 1.2]), pos=pos, a=rng.uniform(0.8, 1.2, 1500))
    o = make_open_oracle(case)
    o.set_threads(8)
    s = make_open_system(case)
    x = rng.standard_normal(s.n)
    assert rel_l2(s.atimes_3all(x), o.atimes_nonewald(x)) < TOL
    s.close()


def test_chebyshev_on_the_open_operator(lib, nonewald):
    """The Chebyshev noise of an open system (src/chebyshev.c:163-228 with
    atimes_nonewald_3all) runs on the device operator and equals the host
    Clenshaw recurrence over the oracle's product."""
    from libstokes_gb300 import abi
    case = nonewald["n200_v2_mono"]
    s = make_open_system(case)
    n = s.n
    rng = np.random.default_rng(4)
    y = rng.standard_normal(n)
    ncheb, e0, e1 = 12, 0.05, 3.0
    a = np.zeros(ncheb)
    f = abi.FUNC1(lambda t: 1.0 / np.sqrt(t))
    lib.chebyshev_coef(ncheb, f, e0, e1, abi._d(a))
    z = np.zeros(n)
    fp = C.cast(lib.atimes_nonewald_3all, C.c_void_p)
    lib.chebyshev_eval_atimes(ncheb, abi._d(a), n, abi._d(y), abi._d(z), e0, e1, fp,
                              C.cast(s.sp, C.c_void_p))
    abi.raise_if_failed()
    # the recurrence of src/chebyshev.c:163-228 over the oracle's product
    o = make_open_oracle(case)
    da, db = 2.0 / (e1 - e0), -(e1 + e0) / (e1 - e0)
    b1, b2 = np.zeros(n), np.zeros(n)
    for j in range(ncheb - 1, 0, -1):
        b1, b2 = 2 * da * o.atimes_nonewald(b1) + 2 * db * b1 - b2 + a[j] * y, b1
    ref = da * o.atimes_nonewald(b1) + db * b1 - b2 + a[0] * y
    assert rel_l2(z, ref) < 1e-12
    s.close()
