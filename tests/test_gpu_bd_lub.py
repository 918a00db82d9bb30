"""Brownian dynamics with lubrication (BD->flag_lub, src/brownian.c:2352-2560
through solve_mix_3all): each velocity of the mid-point step solves the
lubricated mobility problem (I + M L) u = M f (src/ewald-3f.c:447-490) on
the device.  Checked on a deterministic step (peclet 0: no Brownian force,
constant external forces) against the same step composed from the oracle's
dense mobility matrix and lubrication operator with a dense solve.  The
lubrication noise of BD_calc_FB (flag_lub_B, src/brownian.c:1734-1849, the
Chebyshev form) against the reference's own routine on the same KIrand
stream (tests/golden/lub.npz), and its Lanczos bounds."""
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


def _lub_noise_bd(lib, r, seed, eig, eigl, eps=10.0):
    """struct stokes + struct BD_params of a lubrication-noise fixture:
    flag_lub_B = 1, the Chebyshev form (n_lub > 0), bounds as given (equal
    bounds: estimated by the library)."""
    from libstokes_gb300 import System, abi
    from libstokes_gb300.abi import FUNC1
    ver, n, L, lubmin2, lubmax, nminv, nlub, _ = r["meta"]
    ver, n, nminv, nlub = int(ver), int(n), int(nminv), int(nlub)
    s = System(ver, r["pos"], (L, L, L))
    s.s.lubmin2 = float(lubmin2)
    s.s.lubmax = float(lubmax)
    keep = [np.zeros(3 * n), np.zeros(3 * n), np.zeros(5 * n)]
    dp = abi._dp
    bd = lib.BD_params_init(s.sp, int(seed), keep[0].ctypes.data_as(dp),
                            keep[1].ctypes.data_as(dp), keep[2].ctypes.data_as(dp), None, None,
                            None, 0, 1, 0, 0.0, None, None, 1.0, None, None, None, None, None, 0,
                            1.0, eps, nminv, nlub, 0, 0.0, 0.0, 1e-12)
    bd.contents.flag_lub_B = 1
    bd.contents.eig_minv[0], bd.contents.eig_minv[1] = float(eig[0]), float(eig[1])
    fs = [FUNC1(lambda v: 1.0 / np.sqrt(v)), FUNC1(lambda v: np.sqrt(v))]
    lib.chebyshev_coef(nminv, fs[0], float(eig[0]), float(eig[1]), bd.contents.a_minv)
    bd.contents.eig_lub[0], bd.contents.eig_lub[1] = float(eigl[0]), float(eigl[1])
    if eigl[0] != eigl[1]:
        lib.chebyshev_coef(nlub, fs[1], float(eigl[0]), float(eigl[1]), bd.contents.a_lub)
    return s, bd, keep + fs


def _lub_noise_case(name):
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "lub.npz"))
    return {k[len(name) + 1:]: d[k] for k in d.files if k.startswith(name + "_")}


@pytest.mark.parametrize("name", ["lubnoise_f", "lubnoise_ft"])
def test_calc_fb_lubrication_noise_matches_reference(lib, name):
    """BD_calc_FB with flag_lub_B (z = M^-1/2 y + L^1/2 y_lub, the Chebyshev
    form, src/brownian.c:1597-1849) against the reference's own routine on
    the same KIrand stream and preset bounds (tests/golden/lub.npz)."""
    from libstokes_gb300 import abi
    r = _lub_noise_case(name)
    s, bd, keep = _lub_noise_bd(lib, r, r["meta"][7], r["eig"], r["eigl"])
    z = np.zeros(lib.BD_get_n(s.sp))
    lib.BD_calc_FB(bd, z.ctypes.data_as(abi._dp))
    abi.raise_if_failed()
    err = np.linalg.norm(z - r["z"]) / np.linalg.norm(r["z"])
    assert err < 1e-10, err
    lib.BD_params_free(bd)
    s.close()


@pytest.mark.parametrize("name", ["lubnoise_f", "lubnoise_ft"])
def test_lubrication_noise_bounds_by_lanczos(lib, name):
    """With eig_lub unset, the library estimates the bounds of L by Lanczos
    (the reference calls ARPACK there): they bracket L's spectrum, and a
    second call with the estimated bounds preset gives the same noise."""
    from libstokes_gb300 import abi
    r = _lub_noise_case(name)
    seed = int(r["meta"][7])
    s, bd, keep = _lub_noise_bd(lib, r, seed, r["eig"], (0.0, 0.0))
    z1 = np.zeros(lib.BD_get_n(s.sp))
    lib.BD_calc_FB(bd, z1.ctypes.data_as(abi._dp))
    abi.raise_if_failed()
    e0, e1 = bd.contents.eig_lub[0], bd.contents.eig_lub[1]
    lev = r["lev"]                       # L's extreme eigenvalues (dense, reference)
    # the largest Ritz value converges first; the smallest may not in the
    # Lanczos steps, so only its sign and order are checked
    assert 0.0 <= e0 < e1 and lev[1] <= e1 < 1.2 * lev[1], (e0, e1, lev)
    lib.BD_params_free(bd)
    s.close()
    s, bd, keep = _lub_noise_bd(lib, r, seed, r["eig"], (e0, e1))
    z2 = np.zeros(lib.BD_get_n(s.sp))
    lib.BD_calc_FB(bd, z2.ctypes.data_as(abi._dp))
    abi.raise_if_failed()
    assert np.linalg.norm(z2 - z1) < 1e-12 * np.linalg.norm(z1)
    lib.BD_params_free(bd)
    s.close()


def test_evolve_mid_with_lubrication_noise(lib):
    """BD_evolve_mid with flag_lub and flag_lub_B: the step runs on the
    device with both noises (the lubrication draws follow the mobility
    draws on the KIrand stream) and differs from the same step without the
    lubrication noise."""
    from libstokes_gb300 import abi
    r = _lub_noise_case("lubnoise_f")
    seed = int(r["meta"][7])
    steps = []
    for flag_b in (1, 0):
        s, bd, keep = _lub_noise_bd(lib, r, seed, r["eig"], r["eigl"])
        bd.contents.flag_lub_B = flag_b
        x = np.ascontiguousarray(r["pos"].reshape(-1).copy())
        done = lib.BD_evolve_mid(0.0, bd, x.ctypes.data_as(abi._dp), None, 1e-4)
        abi.raise_if_failed()
        assert done == 1e-4
        assert np.all(np.isfinite(x))
        steps.append(x - r["pos"].reshape(-1))
        lib.BD_params_free(bd)
        s.close()
    assert np.linalg.norm(steps[0] - steps[1]) > 1e-3 * np.linalg.norm(steps[1])
