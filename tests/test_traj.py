"""Trajectory and checkpoint files (include/stokes_traj.h): the content of
libstokes' NetCDF output (src/stokes-nc.c) in a plain binary file.  Host
code only: round trips bit for bit, the generator state resumes the same
stream, a frame cut short is dropped, and foreign files are refused."""
import ctypes as C
import os

import numpy as np
import pytest


def _frame(lib, np_, nf, rng_state=None, seed=0):
    from libstokes_gb300.abi import TrajFrame, _d
    r = np.random.default_rng(seed)
    arrays = {k: r.standard_normal(w * (nf if k == "xf" else np_))
              for k, w in (("x", 3), ("u", 3), ("o", 3), ("e", 5), ("f", 3), ("t", 3), ("s", 5),
                           ("q", 4), ("xf", 3))}
    fr = TrajFrame()
    fr.time = float(r.uniform(0, 10))
    fr.shear_shift = float(r.uniform(-1, 1))
    for k, v in arrays.items():
        setattr(fr, k, _d(v))
    fr.rng = C.cast(rng_state, C.c_void_p) if rng_state is not None else None
    return fr, arrays


def test_round_trip_every_field(lib, tmp_path):
    from libstokes_gb300 import System
    from libstokes_gb300.abi import TrajFrame, _d
    np_, nf = 7, 3
    pos = np.random.default_rng(1).uniform(0, 9, (np_ + nf, 3))
    s = System(1, pos, (9.0, 9.5, 10.0))
    lib.stokes_set_np(s.sp, np_ + nf, np_)
    a = np.linspace(0.8, 1.2, np_ + nf)
    s.set_radius(a)
    lib.stokes_set_shear(s.sp, 1, 0.7)
    path = str(tmp_path / "run.traj").encode()
    rng = lib.KIrand_init()
    lib.KIrand_init_genrand(rng, 99)
    t = lib.stokes_traj_create(path, np_, nf, 1023, s.sp)
    assert t
    written = []
    for k in range(3):
        fr, arrays = _frame(lib, np_, nf, rng, seed=k)
        assert lib.stokes_traj_append(t, C.byref(fr)) == 0
        written.append((fr.time, fr.shear_shift, arrays))
    lib.stokes_traj_close(t)

    t = lib.stokes_traj_open(path)
    assert t and lib.stokes_traj_nframes(t) == 3
    ni, nfi, ver, fld = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    box, ar, afr = np.zeros(3), np.zeros(np_), np.zeros(nf)
    assert lib.stokes_traj_info(t, C.byref(ni), C.byref(nfi), C.byref(ver), C.byref(fld),
                                _d(box), _d(ar), _d(afr)) == 0
    assert (ni.value, nfi.value, ver.value, fld.value) == (np_, nf, 1, 1023)
    np.testing.assert_array_equal(box, [9.0, 9.5, 10.0])
    np.testing.assert_array_equal(np.concatenate([ar, afr]), a)
    for k in (2, 0, 1):
        time, shift, arrays = written[k]
        out = {key: np.zeros_like(v) for key, v in arrays.items()}
        fr = TrajFrame()
        for key, v in out.items():
            setattr(fr, key, _d(v))
        assert lib.stokes_traj_read(t, k, C.byref(fr)) == 0
        assert fr.time == time and fr.shear_shift == shift
        for key in arrays:
            np.testing.assert_array_equal(out[key], arrays[key], err_msg=key)
    assert lib.stokes_traj_read(t, 3, C.byref(fr)) != 0
    lib.stokes_traj_close(t)
    lib.KIrand_free(rng)
    s.close()


def test_generator_state_resumes_the_stream(lib, tmp_path):
    """All 624 words of the MT19937 state, the index and the saved Gaussian
    deviate: a generator read back continues exactly where the saved one
    was (an odd number of Gaussians leaves a saved deviate)."""
    from libstokes_gb300.abi import TrajFrame
    path = str(tmp_path / "ckpt.traj").encode()
    r = lib.KIrand_init()
    lib.KIrand_init_genrand(r, 4357)
    for _ in range(1001):
        lib.KIrand_Gaussian(r)
    t = lib.stokes_traj_create(path, 0, 0, 512, None)
    fr = TrajFrame()
    fr.rng = C.cast(r, C.c_void_p)
    assert lib.stokes_traj_append(t, C.byref(fr)) == 0
    lib.stokes_traj_close(t)
    ahead = [lib.KIrand_Gaussian(r) for _ in range(777)] + \
            [lib.KIrand_genrand_int32(r) for _ in range(700)]
    r2 = lib.KIrand_init()
    lib.KIrand_init_genrand(r2, 1)
    t = lib.stokes_traj_open(path)
    fr2 = TrajFrame()
    fr2.rng = C.cast(r2, C.c_void_p)
    assert lib.stokes_traj_read(t, 0, C.byref(fr2)) == 0
    lib.stokes_traj_close(t)
    again = [lib.KIrand_Gaussian(r2) for _ in range(777)] + \
            [lib.KIrand_genrand_int32(r2) for _ in range(700)]
    assert again == ahead
    lib.KIrand_free(r)
    lib.KIrand_free(r2)


def test_cut_frame_is_dropped_and_rewritten(lib, tmp_path):
    from libstokes_gb300.abi import TrajFrame, _d
    path = tmp_path / "cut.traj"
    t = lib.stokes_traj_create(str(path).encode(), 5, 0, 1 | 16, None)
    for k in range(3):
        fr, _ = _frame(lib, 5, 0, seed=k)
        assert lib.stokes_traj_append(t, C.byref(fr)) == 0
    lib.stokes_traj_close(t)
    size = os.path.getsize(path)
    with open(path, "r+b") as f:
        f.truncate(size - 17)
    t = lib.stokes_traj_open(str(path).encode())
    assert lib.stokes_traj_nframes(t) == 2
    fr, arrays = _frame(lib, 5, 0, seed=11)
    assert lib.stokes_traj_append(t, C.byref(fr)) == 0
    assert lib.stokes_traj_nframes(t) == 3
    x = np.zeros(15)
    rd = TrajFrame()
    rd.x = _d(x)
    assert lib.stokes_traj_read(t, 2, C.byref(rd)) == 0
    np.testing.assert_array_equal(x, arrays["x"])
    lib.stokes_traj_close(t)
    assert os.path.getsize(path) == size


def test_foreign_files_are_refused(lib, tmp_path):
    p = tmp_path / "other.bin"
    p.write_bytes(b"CDF\x01" + bytes(200))
    assert not lib.stokes_traj_open(str(p).encode())
    assert not lib.stokes_traj_open(str(tmp_path / "missing").encode())
