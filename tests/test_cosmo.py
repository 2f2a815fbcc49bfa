"""Host cosmology (src/cosmo.jl): the tabulated comoving distance against an
adaptive quadrature, and the FP32 density parameters."""
import numpy as np


def test_distance_table_matches_quadrature():
    from baorec import cosmo
    c = cosmo.Cosmology(z_tab_max=10.0, z_tab_num=20001)
    zg, r = c.distance_table()
    assert zg[0] == 0.0 and r[0] == 0.0 and abs(zg[-1] - 10.0) < 1e-12
    for z in (0.05, 0.8, 1.0, 2.5, 9.9):
        i = int(round(z / (zg[1] - zg[0])))
        q = c.comoving_distance(zg[i])
        assert abs(r[i] / q - 1) < 1e-9, (z, r[i], q)
    assert np.all(np.diff(r) > 0)


def test_density_parameters_close_to_one_and_desi_defaults():
    from baorec import cosmo
    for c in (cosmo.Cosmology(), cosmo.DESICosmology()):
        total = float(c.Omega_L0) + float(c.Omega_m0) + float(c.Omega_g0) + float(c.Omega_nu0) + float(c.Omega_k0)
        assert abs(total - 1.0) < 1e-6
        assert abs(float(c.E(0.0)) - 1.0) < 1e-6
    d = cosmo.DESICosmology()
    assert abs(float(d.h) - 0.6736) < 1e-7 and abs(float(d.H0) - 67.36) < 1e-4
