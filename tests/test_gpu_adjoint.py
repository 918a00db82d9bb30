"""Vector-Jacobian product on the GPU (stokes_gpu_vjp) against the CPU oracle
gradient (oracle/oracle_adjoint.cpp), against central differences of the GPU
FP64 product (h = 1e-4), and as the driver of a short gradient descent."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _vjp(lib, s, g, f, box=True):
    n = s.n
    dr = np.zeros(3 * s.s.np)
    db = np.zeros(3)
    L = C.c_double()
    rc = lib.stokes_gpu_vjp(s.sp, _dp(g), _dp(f), _dp(dr), _dp(db) if box else None, C.byref(L))
    assert rc == 0, lib.stokes_gpu_last_error_message()
    return L.value, dr, db


@pytest.mark.parametrize("version,n,phi", [(0, 24, 0.2), (1, 24, 0.2), (1, 40, 0.3)])
def test_vjp_matches_oracle(lib, version, n, phi):
    from libstokes_gb300 import System
    from libstokes_gb300.workloads import rsa_positions
    from oracle.oracle import Oracle
    pos, L = rsa_positions(n, phi, seed=11 + n)
    c = (3, 6)[version]
    rng = np.random.default_rng(n)
    g = rng.standard_normal(c * n)
    f = rng.standard_normal(c * n)
    s = System(version, pos, (L, L, L))
    Lg, dr, db = _vjp(lib, s, g, f)
    o = Oracle(version, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    Lo, dro, dbo = o.vjp(pos, g, f)
    assert abs(Lg - Lo) < 1e-12 * abs(Lo)
    assert rel_l2(dr, dro) < 1e-10
    assert np.abs(db - dbo).max() < 1e-9 * max(1.0, np.abs(dbo).max())
    s.close()


def test_vjp_central_differences(lib):
    """FT, N = 64: spot coordinates and the box against central differences
    (h = 1e-4) of g . M f through the GPU FP64 product."""
    from libstokes_gb300 import System
    from libstokes_gb300.workloads import rsa_positions
    n, c = 64, 6
    pos, L = rsa_positions(n, 0.25, seed=5)
    rng = np.random.default_rng(6)
    g = rng.standard_normal(c * n)
    f = rng.standard_normal(c * n)
    s = System(1, pos, (L, L, L))
    _, dr, db = _vjp(lib, s, g, f)
    xi = s.s.xi
    h = 1e-4

    def loss(p, box=(L, L, L)):
        t = System(1, p, box, xi=xi)
        v = g @ t.atimes(f)
        t.close()
        return v

    for k in rng.choice(3 * n, 12, replace=False):
        p = pos.reshape(-1).copy()
        p[k] += h
        a = loss(p)
        p[k] -= 2 * h
        b = loss(p)
        fd = (a - b) / (2 * h)
        assert abs(dr[k] - fd) < 1e-6 * max(1.0, abs(fd)), (k, dr[k], fd)
    for a in range(3):
        bp, bm = [L, L, L], [L, L, L]
        bp[a] += h
        bm[a] -= h
        fd = (loss(pos, tuple(bp)) - loss(pos, tuple(bm))) / (2 * h)
        assert abs(db[a] - fd) < 1e-6 * max(1.0, abs(fd)), (a, db[a], fd)
    s.close()


def test_gradient_descent_fits_velocity_field(lib):
    """Positions fitted to a target velocity field: loss |M(r) f - u*|^2 with
    the gradient from the VJP at g = 2 (M f - u*); the loss falls."""
    from libstokes_gb300 import System
    from libstokes_gb300.workloads import rsa_positions
    n, c = 128, 6
    pos, L = rsa_positions(n, 0.1, seed=9)
    rng = np.random.default_rng(10)
    f = rng.standard_normal(c * n)
    target_pos = pos + 0.05 * rng.standard_normal(pos.shape)
    t = System(1, target_pos, (L, L, L))
    u_star = t.atimes(f)
    t.close()
    s = System(1, pos, (L, L, L))

    def loss_at(x):
        lib.stokes_set_pos(s.sp, _dp(x))
        r = s.atimes(f) - u_star
        return float(r @ r), r

    x = pos.reshape(-1).copy()
    lv, r = loss_at(x)
    losses = [lv]
    step = 1e-3
    for it in range(10):
        _, dr, _ = _vjp(lib, s, 2.0 * r, f, box=False)
        # backtracking: a descent direction must lower the loss for a small step
        for _ in range(30):
            xn = x - step * dr
            ln, rn = loss_at(xn)
            if ln < lv:
                break
            step *= 0.5
        assert ln < lv, (it, ln, lv)
        x, lv, r = xn, ln, rn
        losses.append(lv)
        step *= 2.0
    assert losses[-1] < 0.9 * losses[0], losses
    s.close()


def _mixed_vjp_ran(lib, s):
    from libstokes_gb300 import abi
    return any(k.startswith("kva_") for k in abi.kernel_profile(lib, s.sp))


@pytest.mark.parametrize("version,n,phi", [(0, 150, 0.05), (1, 150, 0.05)])
def test_mixed_vjp_matches_oracle(lib, version, n, phi):
    """The mixed-precision VJP (FP32 terms, its own split) against the CPU
    oracle's FP64 gradient at libstokes' split: 1e-6 relative L2 on dL/dr,
    1e-6 of the largest on dL/dbox."""
    from libstokes_gb300 import MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    from oracle.oracle import Oracle
    import os
    pos, L = rsa_positions(n, phi, seed=31 + version)
    c = (3, 6)[version]
    rng = np.random.default_rng(40 + version)
    g = rng.standard_normal(c * n)
    f = rng.standard_normal(c * n)
    s = System(version, pos, (L, L, L))
    s.set_precision(MIXED)
    lib.stokes_gpu_kprof_begin(s.sp, 16)
    Lg, dr, db = _vjp(lib, s, g, f)
    assert _mixed_vjp_ran(lib, s)
    o = Oracle(version, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    o.set_threads(os.cpu_count() or 1)
    Lo, dro, dbo = o.vjp(pos, g, f)
    # L = g . M f from the mixed product: 1e-6 of |g| |f| (L itself is a
    # sum of c N terms that cancel)
    assert abs(Lg - Lo) < 1e-6 * np.linalg.norm(g) * np.linalg.norm(f)
    assert rel_l2(dr, dro) < 1e-6, rel_l2(dr, dro)
    # dL/dbox is a sum over every pair and k vector whose terms cancel to
    # about 1e-3 of their size; FP32 terms hold it to a few 1e-6
    assert np.abs(db - dbo).max() < 1e-5 * np.abs(dbo).max(), (db, dbo)
    s.close()


def test_mixed_vjp_ft_n2048_against_fp64(lib):
    """FT, N = 2048, phi 0.25 (the differentiated workload): the mixed VJP
    against the FP64 VJP at 1e-6 (dL/dr relative L2, dL/dbox of the largest)."""
    from libstokes_gb300 import FP64, MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(2048, 0.25, seed=42)
    rng = np.random.default_rng(1)
    g = rng.standard_normal(6 * 2048)
    f = rng.standard_normal(6 * 2048)
    s = System(1, pos, (L, L, L))
    L64, dr64, db64 = _vjp(lib, s, g, f)
    s.set_precision(MIXED)
    lib.stokes_gpu_kprof_begin(s.sp, 16)
    Lm, drm, dbm = _vjp(lib, s, g, f)
    assert _mixed_vjp_ran(lib, s)
    assert abs(Lm - L64) < 1e-6 * np.linalg.norm(g) * np.linalg.norm(f)
    assert rel_l2(drm, dr64) < 1e-6, rel_l2(drm, dr64)
    # the box derivative: a cancelling sum (see test_mixed_vjp_matches_oracle)
    assert np.abs(dbm - db64).max() < 1e-5 * np.abs(db64).max(), (dbm, db64)
    s.set_precision(FP64)
    s.close()
