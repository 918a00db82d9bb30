"""The lubrication correction on the GPU (calc_lub_3f / 3ft / 3fts and the
dense matrices make_matrix_lub_3f / 3ft / 3fts,
src/lub.c:164-768, equal spheres) against the reference's own outputs
(tests/golden/lub.npz: periodic, open, sheared, small-box and
unlimited-range systems) and against the oracle on larger systems; the
refusals (unequal radii, a bad version, an image cube too large); and the
lubricated mobility problem (I + M L) u = M f solved on the device against
a dense solve."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["lub_f_periodic", "lub_ft_periodic", "lub_f_open", "lub_ft_open", "lub_ft_nolimit",
         "lub_f_small_box", "lub_f_shear1", "lub_ft_shear2", "lub_fts_periodic", "lub_fts_open",
         "lub_fts_shear1"]


@pytest.fixture(scope="module")
def lub():
    return np.load(os.path.join(HERE, "golden", "lub.npz"))


def _system(ver, pos, L, periodic, lubmin2, lubmax, mode=0, shift=0.0):
    from libstokes_gb300 import System
    s = System(ver, pos, (L, L, L)) if periodic else System(ver, pos, periodic=False)
    if mode:
        s.set_misc(0.0, mode, shift)
    s.s.lubmin2 = float(lubmin2)
    s.s.lubmax = float(lubmax)
    return s


def _calc(lib, s, ver, u):
    from libstokes_gb300 import abi
    f = np.zeros_like(u)
    rc = lib.stokes_gpu_lub(s.sp, ver, u.ctypes.data_as(abi._dp), f.ctypes.data_as(abi._dp))
    assert rc == abi.STOKES_GPU_OK, lib.stokes_gpu_last_error_message()
    return f


@pytest.mark.parametrize("name", CASES)
def test_lub_against_reference(lib, lub, name):
    ver, n, L, periodic, lubmin2, lubmax, mode, shift = lub[f"{name}_meta"]
    ver = int(ver)
    s = _system(ver, lub[f"{name}_pos"], L, periodic, lubmin2, lubmax, int(mode), shift)
    f = _calc(lib, s, ver, np.ascontiguousarray(lub[f"{name}_u"]))
    assert rel_l2(f, lub[f"{name}_f"]) < 1e-12, rel_l2(f, lub[f"{name}_f"])
    # the drop-in entry point gives the same numbers
    from libstokes_gb300 import abi
    u = np.ascontiguousarray(lub[f"{name}_u"])
    g = np.zeros_like(u)
    (lib.calc_lub_3f, lib.calc_lub_3ft, lib.calc_lub_3fts)[ver](s.sp, u.ctypes.data_as(abi._dp),
                                                               g.ctypes.data_as(abi._dp))
    assert np.array_equal(f, g)
    s.close()


@pytest.mark.parametrize("ver", [0, 1, 2])
def test_lub_large_against_oracle(lib, ver):
    from libstokes_gb300.workloads import rsa_positions
    from oracle.oracle import calc_lub
    pos, L = rsa_positions(1000, 0.35, seed=71 + ver)
    c = (3, 6, 11)[ver]
    u = np.random.default_rng(72).standard_normal(c * 1000)
    s = _system(ver, pos, L, True, 2.0001 ** 2, 3.0)
    f = _calc(lib, s, ver, u)
    fo = calc_lub(ver, pos, (L, L, L), u, lubmin2=2.0001 ** 2, lubmax=3.0)
    assert np.count_nonzero(fo) > 0
    assert rel_l2(f, fo) < 1e-12, rel_l2(f, fo)
    s.close()


def test_lub_refusals(lib):
    from libstokes_gb300 import abi
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(20, 0.2, seed=5)
    s = _system(0, pos, L, True, 0.0, 3.0)
    u = np.ones(60)
    f = np.zeros(60)
    s.set_radius(np.ones(20))
    assert lib.stokes_gpu_lub(s.sp, 0, u.ctypes.data_as(abi._dp),
                              f.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_EINVAL
    assert b"equal spheres" in lib.stokes_gpu_last_error_message()
    s.close()
    s = _system(2, pos, L, True, 0.0, 3.0)
    u = np.ones(220)
    f = np.zeros(220)
    assert lib.stokes_gpu_lub(s.sp, 3, u.ctypes.data_as(abi._dp),
                              f.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_EINVAL
    s.s.lubmax = 1e6                    # an image cube too large to walk
    assert lib.stokes_gpu_lub(s.sp, 2, u.ctypes.data_as(abi._dp),
                              f.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_EINVAL
    assert b"boxes" in lib.stokes_gpu_last_error_message()
    s.close()


@pytest.mark.parametrize("ver", [0, 1])
def test_lubricated_mobility_solve(lib, ver):
    """(I + M L) u = M f on the device (STOKES_GPU_SOLVE_MOB_LUB) against the
    dense solve of the same operator assembled from the GPU's M and L."""
    from libstokes_gb300 import abi
    from libstokes_gb300.workloads import rsa_positions
    n = 60
    c = (3, 6)[ver]
    pos, L = rsa_positions(n, 0.3, seed=81 + ver)
    s = _system(ver, pos, L, True, 2.0001 ** 2, 3.5)
    N = c * n
    M = s.matrix()
    Lm = np.zeros((N, N))
    for k in range(N):
        e = np.zeros(N)
        e[k] = 1.0
        Lm[:, k] = _calc(lib, s, ver, e)
    fvec = np.random.default_rng(3).standard_normal(N)
    b = M @ fvec
    u_dense = np.linalg.solve(np.eye(N) + M @ Lm, b)
    x = np.zeros(N)
    it, res = C.c_int(), C.c_double()
    rc = lib.stokes_gpu_solve(s.sp, abi.SOLVE_MOB_LUB, b.ctypes.data_as(abi._dp),
                              x.ctypes.data_as(abi._dp), 30, 2000, 1e-12, C.byref(it),
                              C.byref(res))
    assert rc == abi.STOKES_GPU_OK, lib.stokes_gpu_last_error_message()
    assert rel_l2(x, u_dense) < 1e-9, rel_l2(x, u_dense)
    s.close()


MAT_CASES = ["lubmat_f_periodic", "lubmat_ft_shear1", "lubmat_ft_nolimit", "lubmat_fts_periodic",
             "lubmat_fts_open", "lubmat_fts_shear2"]


@pytest.mark.parametrize("name", MAT_CASES)
def test_lub_matrix_against_reference(lib, lub, name):
    """The dense L (make_matrix_lub_3f / 3ft / 3fts, src/lub-matrix.c:76-507)
    against the reference's own matrices: periodic, sheared (both modes),
    open, unlimited range; FTS in the extracted form."""
    from libstokes_gb300 import abi
    ver, n, L, periodic, lubmin2, lubmax, mode, shift = lub[f"{name}_meta"]
    ver, n = int(ver), int(n)
    s = _system(ver, lub[f"{name}_pos"], L, periodic, lubmin2, lubmax, int(mode), shift)
    want = lub[f"{name}_mat"]
    mat = np.zeros_like(want)
    assert lib.stokes_gpu_lub_matrix(s.sp, ver, mat.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_OK
    assert np.abs(mat - want).max() < 1e-12 * np.abs(want).max(), np.abs(mat - want).max()
    m2 = np.full_like(want, 7.0)         # fully overwritten
    (lib.make_matrix_lub_3f, lib.make_matrix_lub_3ft, lib.make_matrix_lub_3fts)[ver](
        s.sp, m2.ctypes.data_as(abi._dp))
    assert np.array_equal(mat, m2)
    s.close()


def _extract_map(n):
    """T of libstokes' FTS matrices: mat (T x) = L x per particle
    (src/matrix.c:447-478)."""
    t = np.eye(11)
    t[6:, 6:] = [[2, 0, 0, 0, 1], [0, 2, 0, 0, 0], [0, 0, 2, 0, 0], [0, 0, 0, 2, 0], [1, 0, 0, 0, 2]]
    return np.kron(np.eye(n), t)


@pytest.mark.parametrize("ver", [0, 1, 2])
def test_lub_matrix_matches_operator(lib, ver):
    """At N = 300: mat u (mat T u for FTS) equals L u from the device
    operator, and the device-buffer entry gives the same matrix."""
    import ctypes as C
    import torch
    from libstokes_gb300 import abi
    from libstokes_gb300.workloads import rsa_positions
    n = 300
    c = (3, 6, 11)[ver]
    pos, L = rsa_positions(n, 0.35, seed=111 + ver)
    s = _system(ver, pos, L, True, 2.0001 ** 2, 3.0)
    mat = np.zeros((c * n, c * n))
    assert lib.stokes_gpu_lub_matrix(s.sp, ver, mat.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_OK
    u = np.random.default_rng(112).standard_normal(c * n)
    f = _calc(lib, s, ver, u)
    fm = mat @ (_extract_map(n) @ u if ver == 2 else u)
    assert np.count_nonzero(f) > 0
    assert rel_l2(fm, f) < 1e-12, rel_l2(fm, f)
    d_pos = torch.tensor(pos, dtype=torch.float64, device="cuda").contiguous()
    d_mat = torch.empty((c * n, c * n), dtype=torch.float64, device="cuda")
    rc = lib.stokes_gpu_lub_matrix_dev(s.sp, ver, C.c_void_p(d_pos.data_ptr()),
                                       C.c_void_p(d_mat.data_ptr()), None)
    assert rc == abi.STOKES_GPU_OK
    torch.cuda.synchronize()
    assert np.array_equal(d_mat.cpu().numpy(), mat)
    s.close()
