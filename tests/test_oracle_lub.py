"""The lubrication oracle (oracle/oracle_lub.c) against the reference's own
outputs (tests/golden/lub.npz, made by tests/golden/make_golden.py from the
compiled reference): the 22 lubrication-form two-body functions of
src/two-body-res.c:31 (regenerated here from the Jeffrey-Onishi and Jeffrey
recurrences), the far-field inverses of src/f.c:183, src/ft.c:414 and
src/fts.c:1491, f = L u of src/lub.c:164-768 (F, FT, FTS) on periodic,
open, sheared, small-box and unlimited-range systems, the reference's
dense lubrication matrices (src/lub-matrix.c) as that operator, and its
lubrication noise (BD_calc_FB with flag_lub_B) recomposed from the oracle."""
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


def _clenshaw(a, e0, e1, A, y):
    """z = sum_k a_k T_k(A~) y by the reference's recurrence
    (src/chebyshev.c:163-228), A dense."""
    n = len(a)
    da, db = 2.0 / (e1 - e0), -(e1 + e0) / (e1 - e0)
    b = [np.zeros_like(y), np.zeros_like(y), np.zeros_like(y)]
    for i in range(n - 1):
        j = n - 1 - i
        b[(i + 2) % 3] = 2.0 * da * (A @ b[(i + 1) % 3]) + 2.0 * db * b[(i + 1) % 3] \
            - b[i % 3] + a[j] * y
    i = n - 1
    return da * (A @ b[(i + 1) % 3]) + db * b[(i + 1) % 3] - b[i % 3] + a[0] * y


@pytest.mark.parametrize("name", ["lubnoise_f", "lubnoise_ft"])
def test_lubrication_noise_fixture_recomposed(lib, lub, name):
    """The reference's BD_calc_FB with flag_lub_B (src/brownian.c:1597-1871)
    recomposed from the oracle: y then y_lub from the KIrand stream of the
    seed, z = M^-1/2 y + L^1/2 y_lub by Chebyshev of the oracle's dense M
    and L with the coefficients of the preset bounds, FT reordered to
    [F part, T part]."""
    import ctypes as C
    from libstokes_gb300.abi import FUNC1
    from oracle.oracle import Oracle, calc_lub
    r = {k[len(name) + 1:]: lub[k] for k in lub.files if k.startswith(name + "_")}
    ver, n, L, lubmin2, lubmax, nminv, nlub, seed = r["meta"]
    ver, n, nminv, nlub, seed = int(ver), int(n), int(nminv), int(nlub), int(seed)
    c = (3, 6)[ver]
    pos = r["pos"]
    o = Oracle(ver, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    M = o.matrix()
    Lm = np.zeros((c * n, c * n))
    for k in range(c * n):
        e = np.zeros(c * n)
        e[k] = 1.0
        Lm[:, k] = calc_lub(ver, pos, (L, L, L), e, lubmin2=lubmin2, lubmax=lubmax)
    rng = lib.KIrand_init()
    lib.KIrand_init_genrand(rng, seed)
    y = np.array([lib.KIrand_Gaussian(rng) for _ in range(c * n)])
    ylub = np.array([lib.KIrand_Gaussian(rng) for _ in range(c * n)])
    lib.KIrand_free(rng)
    fs = [FUNC1(lambda v: 1.0 / np.sqrt(v)), FUNC1(lambda v: np.sqrt(v))]
    am = np.zeros(nminv)
    al = np.zeros(nlub)
    dp = C.POINTER(C.c_double)
    lib.chebyshev_coef(nminv, fs[0], float(r["eig"][0]), float(r["eig"][1]), am.ctypes.data_as(dp))
    lib.chebyshev_coef(nlub, fs[1], float(r["eigl"][0]), float(r["eigl"][1]),
                       al.ctypes.data_as(dp))
    zp = _clenshaw(am, r["eig"][0], r["eig"][1], M, y) \
        + _clenshaw(al, r["eigl"][0], r["eigl"][1], Lm, ylub)
    if ver == 1:
        zp = np.concatenate([zp.reshape(n, 6)[:, :3].ravel(), zp.reshape(n, 6)[:, 3:].ravel()])
    # the lubrication part is a large share: the check is not the mobility
    # noise alone
    assert np.linalg.norm(_clenshaw(al, r["eigl"][0], r["eigl"][1], Lm, ylub)) \
        > 0.1 * np.linalg.norm(zp)
    assert rel_l2(zp, r["z"]) < 1e-10, rel_l2(zp, r["z"])
