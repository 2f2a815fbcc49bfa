"""k-space operators: smoothing, overdensity, the iterative step and the
displacement meshes against the oracle (FP32 cuFFT vs FP32 pocketfft)."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, rel_l2, uniform_box, small_lightcone

pytestmark = pytest.mark.gpu

# FP32 FFTs of different libraries: relative L2 tolerance on a mesh
FFT_TOL = 2e-6


def _noise(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, n, n)).astype(F32)


@pytest.mark.parametrize("n,L,R", [(32, 500.0, 15.0), (64, 1000.0, 10.0), (48, 700.0, 20.0)])
def test_smooth_matches_oracle(n, L, R):
    import baorec
    a = _noise(n, n)
    g = np.asfortranarray(a.copy())
    baorec.smooth_(g, R, [L] * 3)
    o = O.smooth(a.copy(), R, [L] * 3)
    assert rel_l2(g, o) < FFT_TOL


@pytest.mark.parametrize("zpass", [0, 1, 2])
def test_smooth_through_z_pass_matches_oracle(zpass):
    """Meshes with 256 z planes smooth through batched xy transforms and the
    fused z pass (four-step 256-point transform, the Gaussian between them):
    all three transform forms match the oracle to the FFT tolerance."""
    import baorec
    from baorec import recon
    shape, bs, R = (32, 48, 256), [400.0, 600.0, 3200.0], 15.0
    a = np.random.default_rng(5).standard_normal(shape).astype(F32)
    ctx = recon._prim_ctx(shape, bs, [0.0, 0.0, 0.0], smoothing_radius=R)
    ctx.call("baorec_set_tune_zpass", zpass)
    g = np.asfortranarray(a.copy())
    baorec.smooth_(g, R, bs)
    ctx.call("baorec_set_tune_zpass", 1)
    o = O.smooth(a.copy(), R, bs)
    assert rel_l2(g, o) < FFT_TOL


def test_smooth_plane_wave_analytic():
    import baorec
    n, L, R = 32, 400.0, 12.0
    x = (np.arange(n) * L / n)
    kx = 2 * np.pi * 3 / L
    a = np.cos(kx * x)[:, None, None] * np.ones((1, n, n))
    g = np.asfortranarray(a.astype(F32))
    baorec.smooth_(g, R, [L] * 3)
    expect = a * np.exp(-0.5 * R * R * kx * kx)
    assert np.abs(g - expect).max() < 1e-5


def test_setup_overdensity_data_matches_oracle():
    import baorec
    n, L = 32, F32(600.0)
    x, y, z, w = uniform_box(60000, L, seed=1)
    rec = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=[0.0] * 3,
                                los=[0.0, 0.0, 1.0])
    d = baorec.zeros_mesh((n, n, n), device=False)
    gx, gy, gz = x.copy(), y.copy(), z.copy()
    baorec.setup_overdensity_(d, rec, gx, gy, gz, w)
    od, _ = O.setup_overdensity(np.zeros((n, n, n), F32), 2.0, 15.0, [L] * 3, [0.0] * 3, x, y, z, w)
    assert rel_l2(d, od) < 5e-5


def test_setup_overdensity_randoms_matches_oracle():
    import baorec
    m = small_lightcone(n_data=20000, rand_factor=5, n_grid=32)
    n = 32
    bs, bm = O.setup_box(m.rx, m.ry, m.rz, 200.0)
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm)
    d = baorec.zeros_mesh((n, n, n), device=False)
    baorec.setup_overdensity_(d, rec, m.x, m.y, m.z, m.w, m.rx, m.ry, m.rz, m.rw)
    od = O.setup_overdensity_randoms(np.zeros((n, n, n), F32), 2.0, 15.0, bs, bm, m.x, m.y, m.z, m.w,
                                     m.rx, m.ry, m.rz, m.rw)
    # δ = (δ_d - αδ_r)/(bαδ_r) where δ_r > thr: FP32 rounding may flip cells
    # that sit on the threshold, and the division amplifies noise where δ_r is
    # small.  Compare away from the threshold, and bound the flipped cells.
    ran, _ = O.cic(np.zeros((n, n, n), F32), m.rx, m.ry, m.rz, m.rw, bs, bm, wrap=False)
    ran = O.smooth(ran, 15.0, bs)
    thr = 0.01 * float(ran.sum(dtype=np.float64)) / len(m.rx)
    safe = ran > 10 * thr
    assert rel_l2(d[safe], od[safe]) < 2e-5
    near = np.abs(ran - thr) <= 1e-3 * thr
    flipped = (d == 0) != (od == 0)
    assert not np.any(flipped & ~near)


@pytest.mark.parametrize("los", [None, (0.0, 0.0, 1.0), (0.6, 0.0, 0.8)])
def test_iterate_matches_oracle(los):
    import baorec
    n, L = 32, 800.0
    rng = np.random.default_rng(4)
    ds = O.smooth(rng.standard_normal((n, n, n)).astype(F32), 20.0, [L] * 3)
    bm = [200.0, -300.0, 100.0]
    rec = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=bm,
                                los=None if los is None else list(los))
    k = O.k_vec((n, n, n), [L] * 3)
    xv = O.x_vec((n, n, n), [L] * 3, bm)
    g = np.asfortranarray(ds.copy())
    o = ds.copy()
    for it in (1, 2, 3):
        baorec.iterate_(g, ds, it, rec)
        o = O.iterate(o, ds, k, it, rec.beta, los=los, xv=xv)
        assert rel_l2(g, o) < 1e-5, it


@pytest.mark.parametrize("method", ["iterative", "multigrid"])
def test_displacement_meshes_match_oracle(method):
    import baorec
    n, L = 32, 700.0
    rng = np.random.default_rng(7)
    fld = O.smooth(rng.standard_normal((n, n, n)).astype(F32), 20.0, [L] * 3)
    cls = baorec.IterativeRecon if method == "iterative" else baorec.MultigridRecon
    rec = cls(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=[0.0] * 3)
    psi = baorec.compute_displacements(np.asfortranarray(fld), rec)
    ref = O.displacement_meshes_iterative(fld, [L] * 3) if method == "iterative" else O.gradient_meshes(fld, [L] * 3)
    for a in range(3):
        assert rel_l2(psi[a].cpu().numpy(), ref[a]) < FFT_TOL * 5


@pytest.mark.parametrize("method,zpass", [("iterative", 1), ("multigrid", 1), ("multigrid", 2), ("multigrid", 0)])
def test_displacement_through_z_pass_matches_oracle(method, zpass):
    """Meshes with 256 z planes: the displacement spectra from one forward z
    transform and three inverse ones (the gradient multiply between them, over
    k² for the iterative method), against the oracle, for each transform form."""
    import baorec
    shape, bs = (32, 48, 256), [400.0, 600.0, 3200.0]
    fld = O.smooth(np.random.default_rng(9).standard_normal(shape).astype(F32), 30.0, bs)
    cls = baorec.IterativeRecon if method == "iterative" else baorec.MultigridRecon
    rec = cls(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=[0.0] * 3)
    ctx = baorec.setup_fft_(rec, shape)
    ctx.call("baorec_set_tune_zpass", zpass)
    psi = baorec.compute_displacements(np.asfortranarray(fld), rec)
    ref = O.displacement_meshes_iterative(fld, bs) if method == "iterative" else O.gradient_meshes(fld, bs)
    for a in range(3):
        assert rel_l2(psi[a].cpu().numpy(), ref[a]) < FFT_TOL * 5
