"""GPU parity of the FP64 path: atimes_ewald_3all, make_matrix_mob_ewald_3all
and their _notbl / matrix-apply variants against the reference's own outputs
(tests/golden) and against the CPU oracle.

Tolerance: 1e-12 relative L2 (the FP64 bar); dense matrices 1e-12 of the
largest entry."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_oracle, make_system, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def test_atimes_golden(lib, products):
    for name, case in products.items():
        s = make_system(case)
        y = s.atimes(case["x"])
        assert rel_l2(y, case["y"]) < TOL, (name, rel_l2(y, case["y"]))
        if "y_notbl" in case:
            s.restore_table()
            y2 = s.atimes(case["x"], notbl=True)
            assert rel_l2(y2, case["y_notbl"]) < TOL, (name, "notbl")
        s.close()


def test_matrix_golden(lib, products):
    for name, case in products.items():
        if "mat" not in case:
            continue
        s = make_system(case)
        m = s.matrix()
        scale = np.abs(case["mat"]).max()
        assert np.abs(m - case["mat"]).max() / scale < TOL, name
        if "mat_notbl" in case:
            m2 = s.matrix(notbl=True)
            assert np.abs(m2 - case["mat_notbl"]).max() / scale < TOL, (name, "notbl")
        # matrix route of the product (src/ewald.c:484-505)
        y = s.atimes_matrix(case["x"])
        assert rel_l2(y, case["y"]) < TOL, (name, "atimes_3all_matrix")
        s.close()


@pytest.mark.parametrize("version", [0, 1, 2])
def test_against_oracle_rsa(lib, version):
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(60, 0.25, seed=11)
    case = dict(meta=np.array([version, L, L, L, 1.0, 1e-12, 0, 0.0, 0.0]), pos=pos)
    o = make_oracle(case)
    s = make_system(case)
    x = np.random.default_rng(3).standard_normal(s.n)
    assert rel_l2(s.atimes(x), o.atimes(x)) < TOL
    s.close()


def test_mono_equals_poly_unit_radius(lib):
    """test/check-ewald-poly.c: the unequal-radius code at a = 1 equals the
    equal-sphere code."""
    from libstokes_gb300 import System
    phi = 0.2
    l = (np.pi / 0.75 / phi) ** (1.0 / 3.0)
    pos = np.array([[0.0, 0.0, 0.0], [l, 0.0, 0.0]])
    for tr in (1.0, 4.0, 10.0):
        s = System(2, pos, (2 * l,) * 3, tratio=tr)
        x = np.ones(s.n)
        y1 = s.atimes(x)
        m1 = s.matrix()
        s.set_radius(np.ones(2))
        y2 = s.atimes(x)
        m2 = s.matrix()
        assert rel_l2(y2, y1) < 2.3e-14 * 10
        assert np.abs(m1 - m2).max() / np.abs(m1).max() < 2e-14 * 10
        s.close()


@pytest.mark.parametrize("version,shear_mode,phi,tol",
                         [(0, 1, 0.2, 6e-14), (1, 1, 0.4, 2e-13), (2, 2, 0.5, 5e-12)])
def test_shear_shift_invariance(lib, version, shear_mode, phi, tol):
    """test/check-ewald-shear.c: shifting by +-L equals no shift."""
    from libstokes_gb300 import System
    l = (np.pi / 0.75 / phi) ** (1.0 / 3.0)
    pos = np.array([[0.0, 0.0, 0.0], [l, 0.0, 0.0]])
    s = System(version, pos, (2 * l, l, l))
    lib.stokes_set_shear(s.sp, shear_mode, 1.0)
    x = np.ones(s.n)
    s.s.shear_shift = 0.0
    y0 = s.atimes(x)
    for sh in (l, -l):
        s.s.shear_shift = sh
        y = s.atimes(x)
        d = np.abs(y - y0) / np.maximum(np.abs(y0), 1.0)
        assert d.max() < tol * 10, (sh, d.max())
    s.close()


def test_timing_fields_and_launch_count(lib, products):
    s = make_system(products["sc8_v2"])
    s.atimes(products["sc8_v2"]["x"])
    t = s.times()
    assert t[0] > 0 and t[1] > 0 and t[2] > 0
    assert abs(s.s.cpu1 - t[0]) < 1e-9
    cnt = C.c_int()
    assert lib.stokes_gpu_last_launches(s.sp, C.byref(cnt)) == 0
    assert cnt.value >= 3
    s.close()


def test_errors_are_reported_not_faulted(lib, products):
    from libstokes_gb300 import abi
    try:
        case = products["sc8_v0"]
        s = make_system(case)
        # wrong n
        x = np.ones(s.n + 3)
        y = np.zeros(s.n + 3)
        lib.atimes_ewald_3all(s.n + 3, abi._d(x), abi._d(y), C.cast(s.sp, C.c_void_p))
        assert lib.stokes_gpu_last_error() == abi.STOKES_GPU_EINVAL
        assert np.isnan(y).all()
        # a lattice-sum entry point on an open system
        s.s.periodic = 0
        y = np.zeros(s.n)
        lib.atimes_ewald_3all(s.n, abi._d(np.ones(s.n)), abi._d(y), C.cast(s.sp, C.c_void_p))
        assert lib.stokes_gpu_last_error() == abi.STOKES_GPU_ENOTPERIODIC
        assert np.isnan(y).all()
        s.s.periodic = 1
        # the context still works afterwards
        y = s.atimes(case["x"])
        assert rel_l2(y, case["y"]) < TOL
        s.close()
    finally:
        lib.stokes_gpu_set_error_mode(1)


def test_device_entry_point(lib, products):
    import torch
    case = products["r12_v2_mono"]
    s = make_system(case)
    dev = torch.device("cuda:0")
    x = torch.tensor(case["x"], dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    pos = torch.tensor(case["pos"], dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream()
    from libstokes_gb300 import check
    check(lib.stokes_gpu_atimes_dev(s.sp, C.c_void_p(pos.data_ptr()), C.c_void_p(x.data_ptr()),
                                    C.c_void_p(y.data_ptr()), C.c_void_p(st.cuda_stream)))
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), case["y"]) < TOL
    s.close()


def test_default_stream_is_ordered(lib):
    """stream = NULL is the legacy default stream: the product is ordered
    after the caller's earlier work on it and before its later work, so a
    result read back on that stream without a device-wide synchronize is
    complete."""
    import torch
    from libstokes_gb300 import check
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(1000, 0.3, seed=2)
    case = dict(meta=np.array([2, L, L, L, 1.0, 1e-12, 0, 0.0, 0.0]), pos=pos)
    s = make_system(case)
    dev = torch.device("cuda:0")
    x = np.random.default_rng(8).standard_normal(s.n)
    y_host = s.atimes(x)
    with torch.cuda.stream(torch.cuda.default_stream(dev)):
        d_pos = torch.tensor(pos, dtype=torch.float64, device=dev)
        # the input is written by a kernel queued on the default stream
        d_x = torch.zeros(s.n, dtype=torch.float64, device=dev)
        d_x += torch.tensor(x, dtype=torch.float64, device=dev)
        for _ in range(2):
            d_y = torch.full_like(d_x, float("nan"))
            check(lib.stokes_gpu_atimes_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                            C.c_void_p(d_x.data_ptr()),
                                            C.c_void_p(d_y.data_ptr()), None))
            y = d_y.cpu().numpy()     # a copy on the default stream
            assert rel_l2(y, y_host) < TOL
            d_m = torch.full((s.n, s.n), float("nan"), dtype=torch.float64, device=dev)
            check(lib.stokes_gpu_matrix_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                            C.c_void_p(d_m.data_ptr()), None))
            assert torch.isfinite(d_m).all().item()
            del d_m
    s.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_pinned_host_buffers(lib, mixed):
    """Pinned host buffers are used in place by the drop-in call: the same
    result as pageable ones (bit for bit: the same kernels), for both
    precisions, over repeated calls (graph replay) and after the inputs
    change in place."""
    import torch
    from libstokes_gb300 import MIXED
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(300, 0.3, seed=4)
    case = dict(meta=np.array([2, L, L, L, 1.0, 1e-12, 0, 0.0, 0.0]), pos=pos)
    s = make_system(case)
    if mixed:
        s.set_precision(MIXED)
    rng = np.random.default_rng(12)
    hx = torch.empty(s.n, dtype=torch.float64).pin_memory()
    hy = torch.empty(s.n, dtype=torch.float64).pin_memory()
    px = C.cast(C.c_void_p(hx.data_ptr()), C.POINTER(C.c_double))
    py = C.cast(C.c_void_p(hy.data_ptr()), C.POINTER(C.c_double))
    for _ in range(3):
        x = rng.standard_normal(s.n)
        hx.numpy()[:] = x
        hy.numpy()[:] = np.nan
        lib.atimes_ewald_3all(s.n, px, py, C.cast(s.sp, C.c_void_p))
        y_pageable = s.atimes(x)
        np.testing.assert_array_equal(hy.numpy(), y_pageable)
    s.close()


@pytest.mark.parametrize("periodic,pinned", [(True, False), (False, False), (True, True)])
def test_mixed_host_positions_follow_moves(lib, periodic, pinned):
    """The mixed host call reads the positions through a pinned mirror of
    sys->pos, or in place when sys->pos is itself pinned: moving the
    particles between calls gives the device entry point's result on the
    new positions, bit for bit (the same kernels on the same values), for
    the Ewald and the free-space sum."""
    import torch
    from conftest import make_open_system
    from libstokes_gb300 import MIXED, check
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(200, 0.2, seed=9)
    case = dict(meta=np.array([1, L, L, L, 1.0, 1e-12, 0, 0.0, 0.0]), pos=pos)
    s = make_system(case) if periodic else make_open_system(dict(meta=np.array([1, 0.0]), pos=pos))
    s.set_precision(MIXED)
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)
    rt = torch.cuda.cudart()
    addr = C.cast(s.sp.contents.pos, C.c_void_p).value
    if pinned:
        assert int(rt.cudaHostRegister(addr, 8 * pos.size, 0)) == 0
    for step in range(3):
        p = pos + 0.05 * step * rng.standard_normal(pos.shape)
        s.set_pos(p)
        x = rng.standard_normal(s.n)
        y_host = s.atimes_3all(x)
        dx = torch.tensor(x, device=dev)
        dy = torch.empty_like(dx)
        dp = torch.tensor(p.ravel(), device=dev)
        check(lib.stokes_gpu_atimes_dev(s.sp, C.c_void_p(dp.data_ptr()), C.c_void_p(dx.data_ptr()),
                                        C.c_void_p(dy.data_ptr()),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(y_host, dy.cpu().numpy())
    if pinned:
        assert int(rt.cudaHostUnregister(addr)) == 0
    s.close()


@pytest.mark.parametrize("version", [0, 1, 2])
def test_rmin_clamp_off_the_reference_split(lib, version):
    """Overlapping spheres under the rmin clamp (src/ewald.c:693-699), one
    pair nearly coincident.  The FP64 product runs at its tuned split and
    the mixed product at its own; both must reproduce the reference's
    clamped sum at libstokes' split (the oracle): 1e-12 and 1e-6."""
    from libstokes_gb300 import MIXED
    rng = np.random.default_rng(30 + version)
    n, L = 150, 14.0
    pos = rng.uniform(0.0, L, (n, 3))
    pos[1] = pos[0] + np.array([0.003, 0.0, 0.002])
    case = dict(meta=np.array([version, L, L, L, 1.0, 1e-12, 0, 0.0, 1.0]), pos=pos)
    o = make_oracle(case)
    s = make_system(case)
    x = rng.standard_normal(s.n)
    yo = o.atimes(x)
    assert rel_l2(s.atimes(x), yo) < TOL
    s.set_precision(MIXED)
    assert rel_l2(s.atimes(x), yo) < 1e-6
    s.close()
