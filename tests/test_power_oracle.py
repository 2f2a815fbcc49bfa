"""Oracle of the power-spectrum multipoles (pypowspec's estimators, absent
here: parity with it is unpinned).  Physical checks of the restatement:
shot noise of a Poisson catalog, and the survey (Yamamoto) estimator
reducing to the box estimator in the plane-parallel limit."""
import numpy as np

import power_oracle as PO


def _blobs(rng, n, L, bm, ncen=150, sig=(6.0, 6.0, 18.0)):
    """Clustered, anisotropic catalog: Gaussian blobs stretched along z."""
    cen = rng.uniform(0, L, (ncen, 3))
    pick = rng.integers(0, ncen, n)
    p = (cen[pick] + rng.normal(size=(n, 3)) * np.asarray(sig)) % L
    return [p[:, a] + bm[a] for a in range(3)]


def test_poisson_catalog_is_shot_noise():
    rng = np.random.default_rng(0)
    L, n, N = 500.0, 32, 40000
    x, y, z = (rng.uniform(0, L, N) for _ in range(3))
    k, p0, p2, p4, nm, shot, _ = PO.multipoles("box", (n,) * 3, [L] * 3, [0.0] * 3, (x, y, z, None), mas="tsc",
                                               interlace=True, dk=0.02, nbins=8)
    assert abs(shot - L ** 3 / N) / shot < 1e-12
    sig = shot * np.sqrt(2.0 / nm)
    assert np.all(np.abs(p0) < 5 * sig), (p0 / sig)
    assert np.all(np.abs(p2) < 5 * 5 * sig)


def test_survey_estimator_reduces_to_box_far_away():
    """The box placed 1e5 Mpc/h along z: r̂ = ẑ to 2.5e-3 across it, so the
    Yamamoto multipoles equal the box estimator's with LOS z (randoms with
    n(z) = the mean data density give the same normalisation)."""
    rng = np.random.default_rng(1)
    L, n = 500.0, 32
    bm = [-L / 2, -L / 2, 1e5]
    x, y, z = _blobs(rng, 30000, L, bm)
    rx, ry, rz = (rng.uniform(0, L, 150000) + b for b in bm)
    nbar = len(x) / L ** 3
    kw = dict(mas="cic", dk=0.02, nbins=8)
    sv = PO.multipoles("survey", (n,) * 3, [L] * 3, bm, (x, y, z, None), (rx, ry, rz, None),
                       rnz=np.full(len(rx), nbar), **kw)
    bx = PO.multipoles("box", (n,) * 3, [L] * 3, bm, (x, y, z, None), (rx, ry, rz, None), **kw)
    np.testing.assert_array_equal(sv[4], bx[4])
    assert abs(sv[6] - bx[6]) / bx[6] < 1e-12          # normalisation
    for l in (1, 2, 3):
        scale = np.abs(bx[1]).max()
        assert np.abs(sv[l] - bx[l]).max() < 2e-2 * scale, (l, np.abs(sv[l] - bx[l]).max() / scale)
    # blobs stretched along z carry less power along k_z (a finger-of-god
    # shape): a clearly negative quadrupole
    assert bx[2][1:4].max() < -0.1 * bx[1][1:4].max()
