"""Mixed-precision product against the FP64 path on the same inputs.

Bar: relative L2 error <= 1e-6 (the mixed-path tolerance).  The FP64 path is
itself pinned to the reference at 1e-12 (test_gpu_products.py)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-6


def _pair(version, n, phi, seed=1, shear=(0, 0.0)):
    from libstokes_gb300 import FP64, MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=seed)
    x = np.random.default_rng(seed + 100).standard_normal((3, 6, 11)[version] * n)
    a = System(version, pos, (L, L, L))
    b = System(version, pos, (L, L, L))
    for s in (a, b):
        s.set_misc(0.0, *shear)
    a.set_precision(FP64)
    b.set_precision(MIXED)
    return a, b, x


@pytest.fixture(params=["tc", "simt"])
def kspace(request, monkeypatch):
    """Reciprocal space on the tensor cores (default) and on the SIMT path."""
    monkeypatch.setenv("LIBSTOKES_GB300_KSPACE", request.param)
    return request.param


@pytest.mark.parametrize("version,n,phi", [(0, 200, 0.2), (1, 300, 0.25), (2, 200, 0.3),
                                           (2, 1000, 0.3), (0, 1500, 0.2)])
def test_mixed_accuracy(lib, kspace, version, n, phi):
    a, b, x = _pair(version, n, phi)
    y64 = a.atimes(x)
    ymx = b.atimes(x)
    err = rel_l2(ymx, y64)
    assert err < TOL, err
    a.close()
    b.close()


@pytest.mark.parametrize("version,mode,shift", [(0, 1, 3.1), (2, 2, -4.4), (1, 1, 0.0)])
def test_mixed_shear(lib, kspace, version, mode, shift):
    a, b, x = _pair(version, 300, 0.2, seed=4, shear=(mode, shift))
    err = rel_l2(b.atimes(x), a.atimes(x))
    assert err < TOL, err
    a.close()
    b.close()


@pytest.mark.parametrize("version,box", [(2, (1.0, 1.3, 0.8)), (1, (0.7, 1.0, 1.45)),
                                         (0, (1.5, 0.75, 1.0))])
def test_mixed_rectangular_box(lib, kspace, version, box):
    """Unequal box sides: different |m| ranges per axis in the k-space box."""
    from libstokes_gb300 import FP64, MIXED, System
    rng = np.random.default_rng(21)
    n = 240
    L = (4.0 / 3.0 * np.pi * n / 0.06) ** (1.0 / 3.0)
    lx, ly, lz = (L * f for f in box)
    # a loose lattice with jitter keeps the spheres apart
    g = int(np.ceil(n ** (1.0 / 3.0)))
    idx = np.array([(i, j, k) for i in range(g) for j in range(g) for k in range(g)][:n], float)
    pos = (idx + 0.5 + 0.05 * rng.uniform(-1, 1, idx.shape)) * np.array([lx, ly, lz]) / g
    x = rng.standard_normal((3, 6, 11)[version] * n)
    a = System(version, pos.ravel(), (lx, ly, lz))
    b = System(version, pos.ravel(), (lx, ly, lz))
    a.set_precision(FP64)
    b.set_precision(MIXED)
    err = rel_l2(b.atimes(x), a.atimes(x))
    assert err < TOL, err
    a.close()
    b.close()


def test_kspace_paths_agree(lib, monkeypatch):
    """Tensor-core and SIMT reciprocal sums give the same product."""
    from libstokes_gb300 import MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(700, 0.3, seed=33)
    x = np.random.default_rng(34).standard_normal(11 * 700)
    s = System(2, pos, (L, L, L))
    s.set_precision(MIXED)
    monkeypatch.setenv("LIBSTOKES_GB300_KSPACE", "simt")
    y0 = s.atimes(x)
    monkeypatch.setenv("LIBSTOKES_GB300_KSPACE", "tc")
    y1 = s.atimes(x)
    assert rel_l2(y1, y0) < 1e-6
    s.close()


def test_mixed_unwrapped_positions(lib):
    """Positions outside the primary cell give the same product."""
    from libstokes_gb300 import MIXED, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(150, 0.2, seed=8)
    x = np.random.default_rng(9).standard_normal(3 * 150)
    shifted = pos + L * np.random.default_rng(10).integers(-3, 4, pos.shape)
    s1 = System(0, pos, (L, L, L))
    s2 = System(0, shifted, (L, L, L))
    s1.set_precision(MIXED)
    s2.set_precision(MIXED)
    assert rel_l2(s2.atimes(x), s1.atimes(x)) < 1e-6
    s1.close()
    s2.close()


def test_mixed_rejects_unsupported(lib):
    """Slip, and unequal radii under the rmin clamp, stay on the FP64 path."""
    from libstokes_gb300 import MIXED, GPUError, System
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(20, 0.2, seed=2)
    s = System(0, pos, (L, L, L))
    s.set_slip(np.full(20, 0.5))
    s.set_precision(MIXED)
    with pytest.raises(GPUError):
        s.atimes(np.ones(60))
    s.close()
    s = System(0, pos, (L, L, L))
    s.set_radius(np.full(20, 0.9))
    s.set_misc(1.0)
    s.set_precision(MIXED)
    with pytest.raises(GPUError):
        s.atimes(np.ones(60))
    s.close()


@pytest.mark.parametrize("version,n,phi", [(0, 200, 0.2), (1, 160, 0.25), (2, 120, 0.3),
                                           (2, 1000, 0.3)])
def test_mixed_unequal_radii(lib, version, n, phi):
    """Unequal radii (0.6 to 1.0) on the mixed path (FP32 SD-form poly
    scalars in real space, q-weighted structure factors in reciprocal space,
    per-particle self terms) against the FP64 path, which the golden poly
    cases pin to the reference at 1e-12; and the kernels that ran."""
    from libstokes_gb300 import FP64, MIXED, System, abi
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=50 + version)
    a = np.random.default_rng(51 + version).uniform(0.6, 1.0, n)
    x = np.random.default_rng(52).standard_normal((3, 6, 11)[version] * n)
    s = System(version, pos, (L, L, L))
    s.set_radius(a)
    s.set_precision(FP64)
    y64 = s.atimes(x)
    s.set_precision(MIXED)
    lib.stokes_gpu_kprof_begin(s.sp, 16)
    ym = s.atimes(x)
    names = abi.kernel_profile(lib, s.sp)
    assert "mk_backproj_poly" in names, names
    assert rel_l2(ym, y64) < TOL, rel_l2(ym, y64)
    s.close()


def test_mixed_unequal_radii_golden(lib, products):
    """Against the reference's own products for unequal radii."""
    from conftest import make_system
    from libstokes_gb300 import MIXED
    for name in ("r12_v0_poly", "r12_v1_poly", "r12_v2_poly"):
        if name not in products:
            continue
        case = products[name]
        s = make_system(case)
        s.set_precision(MIXED)
        y = s.atimes(case["x"])
        assert rel_l2(y, case["y"]) < TOL, (name, rel_l2(y, case["y"]))
        s.close()


@pytest.mark.parametrize("version,n,phi", [(0, 200, 0.2), (1, 150, 0.25), (2, 120, 0.3)])
def test_mixed_dense_builder(lib, version, n, phi):
    """The split-precision dense builder (k_matrix_f32: FP32 terms, FP64
    entries) against the FP64 builder on the same system: largest entry
    error <= 1e-6 of the largest entry; the matrix route of the product
    (atimes_3all_matrix) against the FP64 product at the mixed bar."""
    a, b, x = _pair(version, n, phi)
    m64 = a.matrix()
    m32 = b.matrix()
    err = np.abs(m32 - m64).max() / np.abs(m64).max()
    assert err < 1e-6, err
    assert err > 0.0              # the FP32 builder, not the FP64 one
    y = b.atimes_matrix(x)
    assert rel_l2(y, a.atimes(x)) < TOL
    a.close()
    b.close()


def test_mixed_dense_builder_golden(lib, products):
    """Against the reference's own matrices (tests/golden), equal spheres."""
    from conftest import make_system
    from libstokes_gb300 import MIXED
    for name in ("sc8_v0", "sc8_v1", "sc8_v2", "r12_v2_mono", "r12_v1_shear1"):
        case = products[name]
        s = make_system(case)
        s.set_precision(MIXED)
        m = s.matrix()
        ref = case["mat"]
        assert np.abs(m - ref).max() / np.abs(ref).max() < 1e-6, name
        s.close()


@pytest.mark.parametrize("version", [0, 1, 2])
@pytest.mark.parametrize("n", [1, 2, 3, 17])
def test_tiny_systems(lib, version, n):
    """One, two, three and seventeen spheres (tensor-core tiles almost all
    padding): FP64 against the oracle at 1e-12, mixed against FP64 at the
    mixed bar, and the split-precision dense builder against the FP64 one."""
    from conftest import make_oracle
    from libstokes_gb300 import FP64, MIXED, System
    rng = np.random.default_rng(40 + n + 10 * version)
    L = 6.0 if n < 10 else 9.0
    pos = np.zeros((n, 3))
    for i in range(n):                      # rejection: centres 2 apart
        while True:
            p = rng.uniform(0, L, 3)
            d = pos[:i] - p
            d -= L * np.rint(d / L)
            if i == 0 or np.min(np.linalg.norm(d, axis=1)) > 2.05:
                pos[i] = p
                break
    case = dict(meta=np.array([version, L, L, L, 1.0, 1e-12, 0, 0.0, 0.0]), pos=pos)
    x = rng.standard_normal((3, 6, 11)[version] * n)
    a = System(version, pos, (L, L, L))
    a.set_precision(FP64)
    y64 = a.atimes(x)
    assert rel_l2(y64, make_oracle(case).atimes(x)) < 1e-12
    b = System(version, pos, (L, L, L))
    b.set_precision(MIXED)
    assert rel_l2(b.atimes(x), y64) < TOL
    m64, m32 = a.matrix(), b.matrix()
    assert np.abs(m32 - m64).max() / np.abs(m64).max() < 1e-6
    a.close()
    b.close()


@pytest.mark.parametrize("n,phi", [(1000, 0.3), (3000, 0.3)])
def test_timed_host_calls_overlap(lib, n, phi):
    """The drop-in call times itself (sys->cpu1..3) with the real space on its
    second stream: over direct launches, the graph capture and its replays,
    with a new x each call, the product matches the FP64 path and the phase
    times add up (total = real + rest, each positive)."""
    a, b, _ = _pair(2, n, phi, seed=17)
    rng = np.random.default_rng(18)
    for call in range(6):
        x = rng.standard_normal(11 * n)
        y = b.atimes(x)
        assert rel_l2(y, a.atimes(x)) < TOL, call
        t = b.times()
        assert t[0] > 0 and t[1] > 0 and t[2] > 0, (call, t)
        assert abs(t[0] - t[1] - t[2]) < 1e-6 * t[0]
        assert (b.s.cpu1, b.s.cpu2, b.s.cpu3) == tuple(t)
    a.close()
    b.close()


@pytest.mark.parametrize("version", [0, 1, 2])
def test_lattice_images_on_request(lib, monkeypatch, version):
    """The real space over lattice images (LIBSTOKES_GB300_MIXED_IMAGES=1, a
    split whose cutoff exceeds half the box) against the FP64 path; the
    default is the minimum-image split, images only for boxes too small."""
    monkeypatch.setenv("LIBSTOKES_GB300_MIXED_IMAGES", "1")
    monkeypatch.setenv("LIBSTOKES_GB300_MIXED_ETA", "6")
    a, b, x = _pair(version, 300, 0.3, seed=23)
    assert rel_l2(b.atimes(x), a.atimes(x)) < TOL
    a.close()
    b.close()
