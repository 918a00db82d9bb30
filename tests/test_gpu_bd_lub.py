"""Brownian dynamics with lubrication (BD->flag_lub, src/brownian.c:2352-2560
through solve_mix_3all): each velocity of the mid-point step solves the
lubricated mobility problem (I + M L) u = M f (src/ewald-3f.c:447-490) on
the device.  Checked on a deterministic step (peclet 0: no Brownian force,
constant external forces) against the same step composed from the oracle's
dense mobility matrix and lubrication operator with a dense solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dense_velocity(ver, pos, L, f, lubmin2, lubmax):
    from oracle.oracle import Oracle, calc_lub
    o = Oracle(ver, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    M = o.matrix()
    n = M.shape[0]
    Lm = np.zeros((n, n))
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        Lm[:, k] = calc_lub(ver, pos, (L, L, L), e, lubmin2=lubmin2, lubmax=lubmax)
    return np.linalg.solve(np.eye(n) + M @ Lm, M @ f)


@pytest.mark.parametrize("ver", [0, 1])
def test_mid_point_step_with_lubrication(lib, ver):
    from libstokes_gb300 import System, abi
    from libstokes_gb300.workloads import rsa_positions
    n = 20
    c = (3, 6)[ver]
    pos, L = rsa_positions(n, 0.30, seed=91 + ver)
    lubmin2, lubmax = 2.0001 ** 2, 3.5
    s = System(ver, pos, (L, L, L))
    s.s.lubmin2 = lubmin2
    s.s.lubmax = lubmax
    lib.stokes_set_iter(s.sp, b"gmres", 4000, 40, 1e-14, 0, None)
    rng = np.random.default_rng(5)
    F = rng.standard_normal(3 * n)
    T = np.zeros(3 * n)
    E = np.zeros(5 * n)
    dp = abi._dp
    bd = lib.BD_params_init(s.sp, 7, F.ctypes.data_as(dp), T.ctypes.data_as(dp),
                            E.ctypes.data_as(dp), None, None, None, 0, 1, 0, 0.0, None, None,
                            1.0, None, None, None, None, None, 0, 0.0, 1.0, 20, 0, 0, 0.0, 0.0,
                            1e-12)
    x = np.ascontiguousarray(pos.reshape(-1).copy())
    dt = 0.02
    done = lib.BD_evolve_mid(0.0, bd, x.ctypes.data_as(dp), None, dt)
    abi.raise_if_failed()
    assert done == dt
    # the same step, densely
    f = np.zeros(c * n)
    for i in range(n):
        f[c * i:c * i + 3] = F[3 * i:3 * i + 3]
    u1 = _dense_velocity(ver, pos, L, f, lubmin2, lubmax)
    xmid = pos + 0.5 * dt * u1.reshape(n, c)[:, :3]
    u2 = _dense_velocity(ver, xmid, L, f, lubmin2, lubmax)
    xnew = pos + dt * u2.reshape(n, c)[:, :3]
    disp = x.reshape(n, 3) - pos
    want = xnew - pos
    assert np.linalg.norm(disp - want) < 1e-9 * np.linalg.norm(want), (
        np.linalg.norm(disp - want) / np.linalg.norm(want))
    lib.BD_params_free(bd)
    s.close()
    # lubrication changes the step (the check is not vacuous): against the
    # same step with u = M f
    from oracle.oracle import Oracle
    o = Oracle(ver, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    xm = pos + 0.5 * dt * (o.matrix() @ f).reshape(n, c)[:, :3]
    o2 = Oracle(ver, xm, (L, L, L))
    o2.set_split(o2.xi_by_tratio(1.0), 1e-12)
    free = dt * (o2.matrix() @ f).reshape(n, c)[:, :3]
    assert np.linalg.norm(free - want) > 1e-2 * np.linalg.norm(want)
