"""The lubrication oracle (oracle/oracle_lub.c) against the reference's own
outputs (tests/golden/lub.npz, made by tests/golden/make_golden.py from the
compiled reference): the 22 lubrication-form two-body functions of
src/two-body-res.c:31 (regenerated here from the Jeffrey-Onishi and Jeffrey
recurrences), the far-field inverses of src/f.c:183, src/ft.c:414 and
src/fts.c:1491, f = L u of src/lub.c:164-768 (F, FT, FTS) on periodic,
open, sheared, small-box and unlimited-range systems, and the reference's
dense lubrication matrices (src/lub-matrix.c) as that operator."""
import os

import numpy as np
import pytest

from conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lub():
    return np.load(os.path.join(HERE, "golden", "lub.npz"))


def test_two_body_functions(lub):
    from oracle.oracle import lub_minv, lub_res2b
    for q, s in enumerate(lub["grid_s"]):
        mine = lub_res2b(s)
        ref = lub["grid_res2b"][q][:22]
        # a function can be small against its singular parts: scale by those
        scale = np.maximum(np.abs(ref), 1e-3)
        assert np.all(np.abs(mine - ref) <= 2e-12 * scale), (s, mine - ref)
        assert np.allclose(lub_minv(0, s), lub["grid_minv_f"][q], rtol=1e-13, atol=1e-15)
        assert np.allclose(lub_minv(1, s), lub["grid_minv_ft"][q], rtol=1e-13, atol=1e-15)
        ref = lub["grid_minv_fts"][q]
        assert np.all(np.abs(lub_minv(2, s) - ref) <= 1e-12 * np.maximum(np.abs(ref), 1e-3)), s


CASES = ["lub_f_periodic", "lub_ft_periodic", "lub_f_open", "lub_ft_open", "lub_ft_nolimit",
         "lub_f_small_box", "lub_f_shear1", "lub_ft_shear2", "lub_fts_periodic", "lub_fts_open",
         "lub_fts_shear1"]


@pytest.mark.parametrize("name", CASES)
def test_calc_lub(lub, name):
    from oracle.oracle import calc_lub
    ver, n, L, periodic, lubmin2, lubmax, mode, shift = lub[f"{name}_meta"]
    f = calc_lub(int(ver), lub[f"{name}_pos"], (L, L, L) if periodic else None,
                 lub[f"{name}_u"], lubmin2=lubmin2, lubmax=lubmax, shear_mode=int(mode),
                 shear_shift=shift)
    ref = lub[f"{name}_f"]
    assert np.linalg.norm(ref) > 0.0
    assert rel_l2(f, ref) < 1e-12, rel_l2(f, ref)


MAT_CASES = ["lubmat_f_periodic", "lubmat_ft_shear1", "lubmat_ft_nolimit", "lubmat_fts_periodic",
             "lubmat_fts_open", "lubmat_fts_shear2"]


@pytest.mark.parametrize("name", MAT_CASES)
def test_dense_matrix_is_the_operator(lub, name):
    """The reference's dense lubrication matrices (src/lub-matrix.c:76-507)
    are the columns of the oracle's L for F and FT, and for FTS the oracle's
    L in libstokes' extracted form, mat (T u) = L u with T per particle
    (2 E0 + E4, 2 E1, 2 E2, 2 E3, E0 + 2 E4), src/matrix.c:447-478."""
    from oracle.oracle import calc_lub
    ver, n, L, periodic, lubmin2, lubmax, mode, shift = lub[f"{name}_meta"]
    ver, n = int(ver), int(n)
    c = (3, 6, 11)[ver]
    want = lub[f"{name}_mat"]
    cols = np.zeros_like(want)
    for k in range(c * n):
        e = np.zeros(c * n)
        e[k] = 1.0
        cols[:, k] = calc_lub(ver, lub[f"{name}_pos"], (L, L, L) if periodic else None, e,
                              lubmin2=lubmin2, lubmax=lubmax, shear_mode=int(mode),
                              shear_shift=shift)
    if ver == 2:
        t = np.eye(11)
        t[6:, 6:] = [[2, 0, 0, 0, 1], [0, 2, 0, 0, 0], [0, 0, 2, 0, 0], [0, 0, 0, 2, 0],
                     [1, 0, 0, 0, 2]]
        got = want @ np.kron(np.eye(n), t)
    else:
        got = want
    assert np.abs(want).max() > 0.0
    assert np.abs(got - cols).max() < 1e-12 * np.abs(cols).max(), np.abs(got - cols).max()


def test_product_coefficients_match_the_oracle():
    """The library's own host-side generation of the series coefficients
    (double precision, libstokes_gb300/csrc/lub.cu) against the oracle's
    (long double): no GPU needed."""
    import ctypes as C
    from libstokes_gb300 import abi
    from oracle.oracle import Oracle
    lib = abi.load()
    mine = np.zeros(22 * 26)
    assert lib.stokes_gpu_lub_coefficients(mine.ctypes.data_as(abi._dp)) == 0
    L = Oracle.lib()
    ref = np.zeros(22 * 26)
    L.oracle_lub_coef.argtypes = [abi._dp]
    L.oracle_lub_coef(ref.ctypes.data_as(abi._dp))
    mine, ref = mine.reshape(22, 26), ref.reshape(22, 26)
    # the terms are c_m / s^(2m) with s >= 2: compare each coefficient's
    # contribution at contact (the difference of the two precisions is below
    # 1e-15 there; in the coefficients it reaches 3e-11 of the largest, high
    # orders of x11a, from the cancellation against the singular part)
    for g in range(22):
        for m in range(26):
            assert abs(mine[g, m] - ref[g, m]) * 0.25 ** m <= 1e-15, (g, m)
