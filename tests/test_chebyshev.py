"""Chebyshev routines (src/chebyshev.c) against the reference's outputs.

Host-only parts (coefficients, scalar evaluation, generic-operator Clenshaw)
run on the CPU; chebyshev_eval_atimes on the Ewald operator keeps every
product on the GPU and is marked gpu."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2


def _funcs():
    from libstokes_gb300.abi import FUNC1
    return {0: FUNC1(lambda x: 1.0 / np.sqrt(x)), 1: FUNC1(lambda x: np.sqrt(x))}


def test_coef_and_eval(lib, cheb_golden):
    from libstokes_gb300.abi import _d
    g = cheb_golden
    fs = _funcs()
    q = 0
    while f"c{q}_args" in g.files:
        nc, which, x0, x1 = g[f"c{q}_args"]
        nc = int(nc)
        a = np.zeros(nc)
        lib.chebyshev_coef(nc, fs[int(which)], x0, x1, _d(a))
        np.testing.assert_allclose(a, g[f"c{q}_a"], rtol=0, atol=1e-14 * np.abs(a).max())
        for x, ref in zip(g[f"c{q}_xs"], g[f"c{q}_eval"]):
            v = lib.chebyshev_eval(nc, _d(a), x0, x1, float(x))
            v2 = lib.chebyshev_eval_(nc, _d(a), x0, x1, float(x))
            assert abs(v - ref) <= 1e-13 * max(1.0, abs(ref))
            assert abs(v2 - ref) <= 1e-12 * max(1.0, abs(ref))
        q += 1


def test_cheb_accuracy_like_reference():
    """test/check-chebyshev.c: 100-term fits of smooth functions reproduce
    them to 1e-10 (host-only)."""
    import libstokes_gb300 as L
    from libstokes_gb300.abi import FUNC1, _d
    lib = L.load()
    for fn in (np.cos, np.sin, np.sqrt):
        f = FUNC1(lambda x, fn=fn: float(fn(x)))
        a = np.zeros(100)
        lib.chebyshev_coef(100, f, 0.5, 3.0, _d(a))
        for x in np.linspace(0.5, 3.0, 100):
            assert abs(lib.chebyshev_eval(100, _d(a), 0.5, 3.0, x) - fn(x)) < 1e-10


def test_eval_atimes_generic_operator(lib, cheb_golden):
    """Host operator through a function pointer (the reference's own path)."""
    from libstokes_gb300.abi import ATIMES, _d
    g = cheb_golden
    M = np.ascontiguousarray(g["dense_M"])
    n = M.shape[0]

    def op(nn, x, y, ud):
        xv = np.ctypeslib.as_array(x, (nn,))
        yv = np.ctypeslib.as_array(y, (nn,))
        yv[:] = M @ xv

    cb = ATIMES(op)
    a = np.ascontiguousarray(g["dense_a"])
    y = np.ascontiguousarray(g["dense_y"])
    z = np.zeros(n)
    e0, e1 = g["dense_e"]
    lib.chebyshev_eval_atimes(len(a), _d(a), n, _d(y), _d(z), e0, e1,
                              C.cast(cb, C.c_void_p), None)
    assert rel_l2(z, g["dense_z"]) < 1e-13
    err = lib.chebyshev_error_minvsqrt(n, _d(y), _d(z), C.cast(cb, C.c_void_p), None)
    assert abs(err - g["dense_err"][0]) < 1e-12


@pytest.mark.gpu
def test_eval_atimes_ewald_on_device(lib, cheb_golden):
    from libstokes_gb300 import System
    from libstokes_gb300.abi import _d
    g = cheb_golden
    s = System(0, g["ewald_pos"], tuple(g["ewald_box"]))
    a = np.ascontiguousarray(g["ewald_a"])
    y = np.ascontiguousarray(g["ewald_y"])
    z = np.zeros(s.n)
    e0, e1 = g["ewald_e"]
    fp = C.cast(lib.atimes_ewald_3all, C.c_void_p)
    lib.chebyshev_eval_atimes(len(a), _d(a), s.n, _d(y), _d(z), e0, e1, fp,
                              C.cast(s.sp, C.c_void_p))
    assert rel_l2(z, g["ewald_z"]) < 1e-12
    err = lib.chebyshev_error_minvsqrt(s.n, _d(y), _d(z), fp, C.cast(s.sp, C.c_void_p))
    assert abs(err - g["ewald_err"][0]) < 1e-10
    s.close()
