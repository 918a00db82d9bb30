"""Pin the CPU oracle (oracle/oracle_ewald.c) to vectors produced by the
reference library itself (tests/golden/, from tests/golden/make_golden.py).

Tolerance: 1e-13 relative L2 -- both sides are FP64 and differ only in
summation order and in the algebraic arrangement of the pair tensors."""
import numpy as np
import pytest

from conftest import make_open_oracle, make_oracle, rel_l2

TOL = 1e-13


def test_oracle_products(products):
    worst = 0.0
    for name, case in products.items():
        o = make_oracle(case)
        y = o.atimes(case["x"])
        err = rel_l2(y, case["y"])
        worst = max(worst, err)
        assert err < TOL, (name, err)
        if "mat" in case:
            m = o.matrix()
            scale = np.abs(case["mat"]).max()
            assert np.abs(m - case["mat"]).max() / scale < TOL, name
    assert worst < TOL


def test_oracle_setup(setup_golden):
    from oracle.oracle import Oracle
    g = setup_golden
    q = 0
    while f"c{q}_box" in g.files:
        box = tuple(g[f"c{q}_box"])
        tr, eps = g[f"c{q}_tr_eps"]
        o = Oracle(0, np.zeros((1, 3)), box)
        o.set_split(o.xi_by_tratio(tr), eps)
        sp = o.split()
        ref = g[f"c{q}_split"]
        got = np.array([sp["xi"], sp["rmax2"], sp["kmax"], sp["self_a"], sp["self_c"],
                        sp["self_m"], sp["pivol"], sp["nr"]] + list(sp["kmaxxyz"]))
        np.testing.assert_array_equal(got, ref)
        rl, rm = o.table()
        np.testing.assert_array_equal(rl, g[f"c{q}_rl"])
        np.testing.assert_array_equal(rm, g[f"c{q}_rm"])
        q += 1
    assert q >= 5


def test_oracle_atimes_matches_its_matrix(products):
    """The reference's own invariant (test/check-ewald.c:46-195): matrix-free
    product == dense matrix (extracted form for FTS) times x."""
    for name in ("sc8_v0", "sc8_v1", "sc8_v2", "r12_v2_slip", "r12_v1_shear1"):
        case = products[name]
        o = make_oracle(case)
        y1 = o.atimes(case["x"])
        y2 = o.matvec(o.matrix(), case["x"])
        assert rel_l2(y1, y2) < 5e-14, name


@pytest.mark.parametrize("shear_mode", [1, 2])
def test_oracle_shear_invariance(shear_mode):
    """Shift of +-L in the flow direction equals no shift
    (test/check-ewald-shear.c:51-167)."""
    from oracle.oracle import Oracle
    phi = 0.2
    l = (np.pi / 0.75 / phi) ** (1.0 / 3.0)
    pos = np.array([[0.0, 0.0, 0.0], [l, 0.0, 0.0]])
    for v, tol in ((0, 6e-14), (1, 2e-13), (2, 5e-12)):
        o = Oracle(v, pos, (2 * l, l, l))
        o.set_split(o.xi_by_tratio(1.0), 1e-12)
        x = np.ones(o.n)
        o.set_misc(0.0, shear_mode, 0.0)
        y0 = o.atimes(x)
        for sh in (l, -l):
            o.set_misc(0.0, shear_mode, sh)
            y = o.atimes(x)
            d = np.abs(y - y0) / np.maximum(np.abs(y0), 1.0)
            assert d.max() < tol, (v, sh, d.max())


def test_oracle_nonewald(nonewald):
    """The free-space restatement (oracle_atimes_nonewald,
    oracle_matrix_nonewald) against the reference's src/non-ewald.c."""
    for name, case in nonewald.items():
        o = make_open_oracle(case)
        if "x" in case:
            err = rel_l2(o.atimes_nonewald(case["x"]), case["y"])
            assert err < TOL, (name, err)
        if "mat" in case:
            m = o.matrix_nonewald()
            scale = np.abs(case["mat"]).max()
            assert np.abs(m - case["mat"]).max() / scale < TOL, name
            if "x" in case:
                assert rel_l2(o.matvec(m, case["x"]), case["y"]) < TOL, name


def test_nonewald_two_spheres_known_answer(nonewald):
    """Two equal spheres on the z axis at r = 2.5 (test/check-minv.c:412-515,
    test/test-all.c:114): the blocks of the reference's matrix are the
    Rotne-Prager-Yamakawa scalars of Durlofsky, Brady and Bossis (1987),
    written out here independently of both implementations."""
    r = 2.5
    xa12, ya12 = 1.5 / r - 1.0 / r ** 3, 0.75 / r + 0.5 / r ** 3
    yb12 = -0.75 / r ** 2
    xc12, yc12 = 0.75 / r ** 3, -0.375 / r ** 3
    for m in (nonewald["pair_ez"]["mat"], make_open_oracle(nonewald["pair_ez"]).matrix_nonewald()):
        assert m.shape == (22, 22)
        # self: a = 1, c = 3/4 (src/non-ewald.c:342-346)
        assert np.allclose(np.diag(m)[[0, 1, 2]], 1.0, rtol=0, atol=1e-15)
        assert np.allclose(np.diag(m)[[3, 4, 5]], 0.75, rtol=0, atol=1e-15)
        # (U_1 | F_2): ya across e, xa along e
        assert abs(m[0, 11] - ya12) < 1e-15 and abs(m[1, 12] - ya12) < 1e-15
        assert abs(m[2, 13] - xa12) < 1e-15
        # (Omega_1 | T_2): yc across e, xc along e
        assert abs(m[3, 14] - yc12) < 1e-15 and abs(m[5, 16] - xc12) < 1e-15
        # (U_1 | T_2): yb (T x e)
        assert abs(m[0, 15] - yb12) < 1e-15 and abs(m[1, 14] + yb12) < 1e-15
        # the pair sees no other coupling of U_1 to F_2
        assert abs(m[0, 13]) < 1e-15 and abs(m[2, 11]) < 1e-15
