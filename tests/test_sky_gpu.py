"""Catalog coordinates on the device against the oracle's restatement of
examples/lightcone.jl:30-82: sky -> Cartesian, Cartesian -> sky (with the
script's ra convention), FKP weights, round trip and out-of-table inputs."""
import numpy as np
import pytest

import baorec_oracle as O

pytestmark = pytest.mark.gpu


def _catalog(n=200000, seed=3):
    rng = np.random.default_rng(seed)
    ra = (rng.random(n) * 90.0).astype(np.float32)
    dec = np.degrees(np.arcsin(rng.random(n) * np.sin(np.radians(45.0)))).astype(np.float32)
    z = (0.8 + 0.2 * rng.random(n)).astype(np.float32)
    return ra, dec, z


def test_sky_to_cartesian_and_back_match_oracle():
    from baorec import cosmo
    c = cosmo.Cosmology(z_tab_max=10.0)
    zg, r = c.distance_table()
    ra, dec, z = _catalog()
    x, y, zc = cosmo.sky_to_cartesian(ra, dec, z, c)
    h_fwd = float(np.float32(c.H0 / np.float32(100)))
    ox, oy, oz = O.sky_to_cartesian(ra, dec, z, zg, r, h_fwd)
    # FP32 trigonometry of two libraries: a few ulps of a ~2000 Mpc/h coordinate
    for a, b in ((x, ox), (y, oy), (zc, oz)):
        assert np.max(np.abs(a - b)) < 1e-3
    ra2, dec2, z2 = cosmo.cartesian_to_sky(x, y, zc, c)
    ora, odec, oz2 = O.cartesian_to_sky(x, y, zc, zg, r, float(np.float32(c.h)))
    assert np.max(np.abs(ra2 - ora)) < 1e-4 and np.max(np.abs(dec2 - odec)) < 1e-4
    assert np.max(np.abs(z2 - oz2)) < 1e-6
    # the script's longitude convention: ra - 360 in (-360, 0]
    assert np.all(ra2 <= 0.0) and np.max(np.abs((ra2 + 360.0) - ra)) < 1e-3
    assert np.max(np.abs(dec2 - dec)) < 1e-3
    # round trip of the redshift (h / (H0/100) differ by at most an ulp)
    assert np.max(np.abs(z2 - z)) < 1e-5


def test_device_arrays_and_fkp():
    import torch
    from baorec import cosmo
    c = cosmo.DESICosmology(z_tab_max=3.0)
    ra, dec, z = _catalog(5000, seed=8)
    out_h = cosmo.sky_to_cartesian(ra, dec, z, c)
    out_d = cosmo.sky_to_cartesian(*(torch.from_numpy(v).cuda() for v in (ra, dec, z)), c)
    for a, b in zip(out_h, out_d):
        np.testing.assert_array_equal(a, b.cpu().numpy())
    nz = (np.random.default_rng(1).random(5000) * 1e-3).astype(np.float32)
    np.testing.assert_array_equal(cosmo.fkp_weights(nz, 1e4), O.fkp_weights(nz, 1e4))


def test_redshift_outside_table_raises_bounds_error():
    from baorec import cosmo
    from baorec._lib import BoundsError
    c = cosmo.Cosmology(z_tab_max=1.0, z_tab_num=1001)
    ra, dec, z = _catalog(100, seed=2)
    z[5] = np.float32(1.5)
    with pytest.raises(BoundsError):
        cosmo.sky_to_cartesian(ra, dec, z, c)
