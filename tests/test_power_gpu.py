"""Power-spectrum multipoles on the GPU against the oracle's restatement of
the same estimators (box: CIC/TSC, interlacing, randoms; survey: Yamamoto
l = 0, 2, 4), on host and device catalogs, and the error cases."""
import numpy as np
import pytest

import power_oracle as PO

pytestmark = pytest.mark.gpu


def _blobs(rng, n, L, bm, ncen=120, sig=(6.0, 6.0, 16.0)):
    cen = rng.uniform(0, L, (ncen, 3))
    pick = rng.integers(0, ncen, n)
    p = (cen[pick] + rng.normal(size=(n, 3)) * np.asarray(sig)) % L
    return [(p[:, a] + bm[a]).astype(np.float32) for a in range(3)]


def _check(got, ref, name):
    k, mp, nm = got["k"], got["multipoles"], got["nmodes"]
    np.testing.assert_array_equal(nm, ref[4])
    np.testing.assert_allclose(k, ref[0], rtol=1e-6)
    assert abs(got["shot_noise"] - ref[5]) <= 1e-9 * ref[5]
    assert abs(got["norm"] - ref[6]) <= 1e-9 * ref[6]
    scale = np.abs(ref[1]).max()
    for l in range(3):
        err = np.abs(mp[:, l] - ref[1 + l]).max()
        assert err < 2e-4 * scale, (name, l, err / scale)


@pytest.mark.parametrize("mas,interlace", [("cic", False), ("tsc", True)])
def test_box_data_only(mas, interlace):
    from baorec import power
    rng = np.random.default_rng(3)
    L, n = 600.0, 48
    x, y, z = _blobs(rng, 40000, L, [0.0] * 3)
    w = rng.uniform(0.5, 1.5, len(x)).astype(np.float32)
    kw = dict(mas=mas, interlace=interlace, kmin=0.0, bin_size=0.02, los=(0.0, 0.6, 0.8))
    got = power.compute_auto_box(x, y, z, w, box_size=L, grid_size=n, **kw)
    nb = len(got["k"])
    ref = PO.multipoles("box", (n,) * 3, [L] * 3, [0.0] * 3, (x, y, z, w), mas=mas, interlace=interlace,
                        los=kw["los"], dk=0.02, nbins=nb)
    _check(got, ref, "box")


def test_box_with_randoms_device_arrays():
    import torch
    from baorec import power
    rng = np.random.default_rng(4)
    L, n = 500.0, 32
    bm = [100.0, -50.0, 0.0]
    x, y, z = _blobs(rng, 20000, L, bm)
    rx, ry, rz = ((rng.uniform(0, L, 60000) + b).astype(np.float32) for b in bm)
    kw = dict(box_size=L, box_min=bm, grid_size=n, mas="tsc", interlace=True, bin_size=0.025)
    host = power.compute_auto_box_rand(x, y, z, None, rx, ry, rz, None, **kw)
    dev = power.compute_auto_box_rand(*[torch.from_numpy(a).cuda() for a in (x, y, z)], None,
                                      *[torch.from_numpy(a).cuda() for a in (rx, ry, rz)], None, **kw)
    ref = PO.multipoles("box", (n,) * 3, [L] * 3, bm, (x, y, z, None), (rx, ry, rz, None), mas="tsc",
                        interlace=True, dk=0.025, nbins=len(host["k"]))
    _check(host, ref, "box+randoms")
    # float atomics paint in any order: same bins, multipoles to FP32 rounding
    np.testing.assert_array_equal(dev["nmodes"], host["nmodes"])
    np.testing.assert_allclose(dev["multipoles"], host["multipoles"], rtol=0,
                               atol=1e-5 * np.abs(host["multipoles"]).max())


def test_survey_multipoles():
    from baorec import power
    rng = np.random.default_rng(5)
    L, n = 400.0, 32
    bm = [300.0, 200.0, 100.0]                         # observer at the origin, outside the box
    x, y, z = _blobs(rng, 30000, L, bm)
    rx, ry, rz = ((rng.uniform(0, L, 120000) + b).astype(np.float32) for b in bm)
    nbar = len(x) / L ** 3
    w = rng.uniform(0.5, 1.0, len(x)).astype(np.float32)
    rw = rng.uniform(0.5, 1.0, len(rx)).astype(np.float32)
    rnz = np.full(len(rx), nbar, np.float32)
    got = power.compute_auto_lc(x, y, z, w, None, rx, ry, rz, rw, rnz, box_size=L, box_min=bm, grid_size=n,
                                mas="cic", bin_size=0.02)
    ref = PO.multipoles("survey", (n,) * 3, [L] * 3, bm, (x, y, z, w), (rx, ry, rz, rw), rnz=rnz, mas="cic",
                        dk=0.02, nbins=len(got["k"]))
    _check(got, ref, "survey")


def test_errors():
    from baorec import _lib, power
    rng = np.random.default_rng(6)
    L, n = 400.0, 16
    x, y, z = (rng.uniform(0, L, 1000).astype(np.float32) for _ in range(3))
    rx, ry, rz = (rng.uniform(0, L, 3000).astype(np.float32) for _ in range(3))
    rnz = np.full(3000, 1e-3, np.float32)
    x[5] = L + 50.0                                     # outside the survey box
    with pytest.raises(_lib.BoundsError):
        power.compute_auto_lc(x, y, z, None, None, rx, ry, rz, None, rnz, box_size=L, box_min=0.0, grid_size=n)
    with pytest.raises(_lib.BaorecError):               # the survey needs randoms
        power.multipoles(x, y, z, geometry="survey", box_size=L, grid_size=n)
    with pytest.raises(_lib.BaorecError):               # no line of sight
        power.multipoles(x, y, z, box_size=L, grid_size=n, los=(0.0, 0.0, 0.0))
