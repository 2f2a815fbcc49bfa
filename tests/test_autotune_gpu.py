"""Autotuner: it picks valid launch shapes, and the solve and the
deterministic paint give the same results with every tile choice."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, small_lightcone, uniform_box

pytestmark = pytest.mark.gpu


def test_autotune_choices_are_valid_and_results_unchanged():
    import baorec
    n = 64
    m = small_lightcone(n_data=30000, rand_factor=5, n_grid=n, seed=9)
    bs, bm = O.setup_box(m.rx, m.ry, m.rz, 25.0 * 256 / n)
    f = O.setup_overdensity_randoms(np.zeros((n, n, n), F32), 2.0, 15.0, bs, bm, m.x, m.y, m.z, m.w,
                                    m.rx, m.ry, m.rz, m.rw)
    ff = np.asfortranarray(f)
    sols = []
    for tuned in (False, True):
        rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm,
                                    mg_mode="convergent", rtol=1e-6, start="zero")
        ctx = baorec.setup_fft_(rec, (n, n, n))
        if tuned:
            ch = ctx.autotune()
            assert ch["paint_tile"] in (4, 8, 16)
            assert all(t in (-1, 0, 1) for t in ch["tile16_per_level"])
            assert ch["tile16_per_level"][0] in (0, 1)   # 64^3: both tile shapes are valid
        phi = baorec.zeros_mesh((n, n, n), device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        sols.append(O.gradient_meshes(np.asarray(phi, np.float64), bs.astype(np.float64)))
    g0, g1 = sols
    for a in range(3):
        assert np.linalg.norm(g1[a] - g0[a]) / np.linalg.norm(g0[a]) < 2e-5


@pytest.mark.parametrize("tile", [4, 16])
def test_deterministic_paint_independent_of_tile(tile):
    """Fixed-point sums make the painted bits independent of the tile edge."""
    import torch
    import baorec
    from baorec import _lib
    n, npart = 32, 40000
    L = F32(400.0)
    x, y, z, w = uniform_box(npart, L, seed=21)
    rec = baorec.IterativeRecon(bias=1.0, f=0.0, smoothing_radius=0.0, box_size=[L] * 3, box_min=[0.0] * 3)
    ctx = baorec.setup_fft_(rec, (n, n, n))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    meshes = []
    for t in (8, tile):
        ctx.call("baorec_set_tune", t, None)
        rho = torch.zeros(n ** 3, device="cuda")
        px, py, pz, pw = dev(x), dev(y), dev(z), dev(w)
        ctx.call("baorec_cic", rho.data_ptr(), px.data_ptr(), py.data_ptr(), pz.data_ptr(), pw.data_ptr(), npart, 1,
                 _lib.DETERMINISTIC)
        meshes.append(rho.cpu().numpy())
    np.testing.assert_array_equal(meshes[0].view(np.uint32), meshes[1].view(np.uint32))
    assert abs(float(meshes[0].sum(dtype=np.float64)) - float(w.sum(dtype=np.float64))) < 1e-2
