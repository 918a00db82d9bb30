"""Iterative solves on the device (include/stokes_iter.h): libiter's
iter_init / solve_iter / iter_free as libstokes calls them, and the FTS
mobility problem solve_mob_3fts_0 (src/ewald-3fts.c:146-314).

The oracle is a dense LU solve of the operator the reference applies,
assembled column by column from the CPU oracle's product (itself pinned to
the reference's outputs).  FP64 solves run to eps = 1e-11 and agree with
the dense solution to 1e-9 relative L2; the mixed path (GMRES on the mixed
product inside FP64 iterative refinement) runs to 1e-10 and agrees with the
FP64 solution to 1e-9."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_open_oracle, make_open_system, make_oracle, make_system, rel_l2

pytestmark = pytest.mark.gpu


def _threads(o):
    import os
    o.set_threads(os.cpu_count() or 1)
    return o


def _dense(op, n):
    """Matrix of a linear map given as a function of vectors."""
    A = np.zeros((n, n))
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        A[:, k] = op(e)
    return A


def _mob_fts(o, x):
    """(u, o, 0) - M (0, 0, s) for x = (u, o, s) (src/ewald-3fts.c:200-247)."""
    np_ = len(x) // 11
    t = x.reshape(np_, 11).copy()
    t[:, :6] = 0.0
    z = o.atimes(t.ravel())
    y = x.reshape(np_, 11).copy()
    y[:, 6:] = 0.0
    return y.ravel() - z


def _rsa_case(version, n=30, phi=0.2, seed=1, poly=False, slip=False, shear=(0, 0.0), rmin=0.0):
    """Non-overlapping spheres (the mobility is positive definite there;
    random overlapping ones make it indefinite and restarted GMRES stalls,
    as it does on the same matrices in any implementation)."""
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=seed)
    rng = np.random.default_rng(seed)
    case = dict(meta=np.array([version, L, L, L, 1.0, 1e-12, shear[0], shear[1], rmin]), pos=pos)
    if poly:
        case["a"] = rng.uniform(0.8, 1.0, n)
    if slip:
        case["slip"] = rng.uniform(0.0, 0.5, n)
    return case


SOLVE_CASES = {
    "f_mono": dict(version=0), "ft_poly": dict(version=1, poly=True),
    "fts_mono": dict(version=2), "fts_slip": dict(version=2, poly=True, slip=True),
    "fts_shear": dict(version=2, shear=(1, 1.3)), "ft_rmin": dict(version=1, rmin=1.0),
}


def _iter(lib, s, eps, restart=20):
    from libstokes_gb300.abi import IterStruct
    lib.stokes_set_iter(s.sp, b"gmres", 2000, restart, eps, 0, None)
    return C.cast(s.s.it, C.POINTER(IterStruct)).contents


@pytest.mark.parametrize("name", sorted(SOLVE_CASES))
def test_resistance_solve_periodic(lib, name):
    """solve_iter (n, b, x, atimes_3all, sys, sys->it): the call of
    src/ewald-3f.c:94, src/ewald-3ft.c:113 and src/ewald-3fts.c:71."""
    from libstokes_gb300.abi import _d
    case = _rsa_case(**SOLVE_CASES[name])
    s = make_system(case)
    o = _threads(make_oracle(case))
    n = s.n
    b = np.random.default_rng(3).standard_normal(n)
    it = _iter(lib, s, 1e-11)
    x = np.zeros(n)
    lib.solve_iter(n, _d(b), _d(x), C.cast(lib.atimes_3all, C.c_void_p),
                   C.cast(s.sp, C.c_void_p), C.cast(s.s.it, C.c_void_p))
    xr = np.linalg.solve(_dense(o.atimes, n), b)
    assert rel_l2(x, xr) < 1e-9, rel_l2(x, xr)
    assert 0 < it.niter <= 2000 and it.res <= 1e-11
    assert rel_l2(o.atimes(x), b) < 1e-10
    s.close()


@pytest.mark.parametrize("name", ["f_mono", "ft_poly", "fts_slip"])
def test_resistance_solve_open(lib, name):
    from libstokes_gb300.abi import _d
    c = _rsa_case(**SOLVE_CASES[name])
    case = dict(meta=np.array([c["meta"][0], 0.0]), pos=c["pos"])
    for k in ("a", "slip"):
        if k in c:
            case[k] = c[k]
    s = make_open_system(case)
    o = _threads(make_open_oracle(case))
    n = s.n
    b = np.random.default_rng(4).standard_normal(n)
    _iter(lib, s, 1e-11)
    x = np.zeros(n)
    lib.solve_iter(n, _d(b), _d(x), C.cast(lib.atimes_3all, C.c_void_p),
                   C.cast(s.sp, C.c_void_p), C.cast(s.s.it, C.c_void_p))
    xr = np.linalg.solve(_dense(o.atimes_nonewald, n), b)
    assert rel_l2(x, xr) < 1e-9
    s.close()


@pytest.mark.parametrize("name", ["fts_mono", "fts_slip", "n40_fts_phi0.30"])
def test_fts_mobility_problem(lib, products, name):
    """solve_mob_3fts_0: given F, T, E the velocities U, O and stresslet S
    with (U, O, E) = M (F, T, S)."""
    from libstokes_gb300.abi import _d
    case = products[name] if name in products else _rsa_case(**SOLVE_CASES[name])
    s = make_system(case)
    o = _threads(make_oracle(case))
    np_ = s.np
    rng = np.random.default_rng(5)
    f, t, e = rng.standard_normal(3 * np_), rng.standard_normal(3 * np_), rng.standard_normal(5 * np_)
    _iter(lib, s, 1e-11)
    u, om, sl = np.zeros(3 * np_), np.zeros(3 * np_), np.zeros(5 * np_)
    lib.solve_mob_3fts_0(s.sp, None, _d(f), _d(t), _d(e), _d(u), _d(om), _d(sl))
    # dense solve of the same problem
    n = 11 * np_
    x1 = np.zeros((np_, 11))
    x1[:, :3], x1[:, 3:6] = f.reshape(-1, 3), t.reshape(-1, 3)
    ev = np.zeros((np_, 11))
    ev[:, 6:] = e.reshape(-1, 5)
    b = o.atimes(x1.ravel()) - ev.ravel()
    xr = np.linalg.solve(_dense(lambda v: _mob_fts(o, v), n), b).reshape(np_, 11)
    got = np.hstack([u.reshape(-1, 3), om.reshape(-1, 3), sl.reshape(-1, 5)])
    assert rel_l2(got, xr) < 1e-9, rel_l2(got, xr)
    # and the physics: M (F, T, S) = (U, O, E)
    fts = np.hstack([f.reshape(-1, 3), t.reshape(-1, 3), sl.reshape(-1, 5)]).ravel()
    uoe = np.hstack([u.reshape(-1, 3), om.reshape(-1, 3), e.reshape(-1, 5)]).ravel()
    assert rel_l2(o.atimes(fts), uoe) < 1e-9
    s.close()


def test_foreign_operator(lib):
    """solve_iter with the caller's own atimes (the reference's static
    operators of the mixed problems take this route): a non-symmetric dense
    operator called back on host vectors."""
    from libstokes_gb300.abi import _d
    rng = np.random.default_rng(6)
    n = 300
    A = np.eye(n) * 4.0 + 0.3 * rng.standard_normal((n, n)) / np.sqrt(n)
    AT = C.CFUNCTYPE(None, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)

    def atimes(nn, xp, yp, _):
        xv = np.ctypeslib.as_array(xp, shape=(nn,))
        yv = np.ctypeslib.as_array(yp, shape=(nn,))
        yv[:] = A @ xv

    cb = AT(atimes)
    it = lib.iter_init(b"gmres", 500, 30, 1e-12, n, None, 0, 0, None)
    b = rng.standard_normal(n)
    x = np.zeros(n)
    lib.solve_iter(n, _d(b), _d(x), C.cast(cb, C.c_void_p), None, it)
    assert rel_l2(x, np.linalg.solve(A, b)) < 1e-10
    from libstokes_gb300.abi import IterStruct
    st = C.cast(it, C.POINTER(IterStruct)).contents
    assert st.res <= 1e-12 and 0 < st.niter < 500
    lib.iter_free(it)


def test_guess_is_kept_between_solves(lib):
    """stokes_set_iter keeps each solution as the next start vector: the
    same right-hand side again converges with (almost) no iterations."""
    from libstokes_gb300.abi import _d
    case = _rsa_case(1)
    s = make_system(case)
    n = s.n
    b = np.random.default_rng(7).standard_normal(n)
    it = _iter(lib, s, 1e-10)
    x = np.zeros(n)
    op = C.cast(lib.atimes_3all, C.c_void_p)
    lib.solve_iter(n, _d(b), _d(x), op, C.cast(s.sp, C.c_void_p), C.cast(s.s.it, C.c_void_p))
    first = it.niter
    x2 = np.zeros(n)
    lib.solve_iter(n, _d(b), _d(x2), op, C.cast(s.sp, C.c_void_p), C.cast(s.s.it, C.c_void_p))
    assert first > 5 and it.niter <= 1
    assert rel_l2(x2, x) < 1e-10
    s.close()


def test_mixed_precision_solve(lib):
    """N = 500 FTS spheres at phi 0.3: the resistance problem and the FTS
    mobility problem solved on the mixed product inside FP64 iterative
    refinement (the residual from the FP64 product) to 1e-10 against the
    FP64 GMRES solve to 1e-11: the solutions agree to 1e-9 and the refined
    residual is the FP64 one."""
    from libstokes_gb300 import FP64, MIXED, System, check
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(500, 0.3, seed=42)
    s = System(2, pos, (L, L, L))
    b = np.random.default_rng(8).standard_normal(s.n)
    for op in (0, 1):
        res = {}
        for mode, eps in ((FP64, 1e-11), (MIXED, 1e-10)):
            s.set_precision(mode)
            x = np.zeros(s.n)
            it = C.c_int()
            r = C.c_double()
            check(lib.stokes_gpu_solve(s.sp, op, _d(b), _d(x), 30, 3000, eps, C.byref(it),
                                       C.byref(r)))
            assert r.value <= eps and it.value > 0, (op, mode, r.value)
            res[mode] = x
        assert rel_l2(res[MIXED], res[FP64]) < 1e-9, (op, rel_l2(res[MIXED], res[FP64]))
        # the refined solution's residual, with the FP64 product
        s.set_precision(FP64)
        if op == 0:
            assert rel_l2(s.atimes(res[MIXED]), b) < 2e-10
    s.close()
