"""Finite-difference gradient read-out (``BAOREC_GRADIENT_FD``): the device
gradient mesh bit for bit against the oracle, the shifts against the
oracle's restatement of the reference's read_grad_cic (src/mas.jl:388-466),
and the FD displacement against the FFT one on a smooth field."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, uniform_box

pytestmark = pytest.mark.gpu


def _rec(L, bm, gradient):
    import baorec
    return baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=list(L), box_min=list(bm),
                                 gradient=gradient)


def test_fd_gradient_mesh_bit_exact():
    """Non-cubic mesh with different box sides: every component equals the
    oracle's FP32 central differences, periodic wrap included."""
    import baorec
    shape = (32, 40, 48)
    L = [F32(640.0), F32(500.0), F32(720.0)]
    rng = np.random.default_rng(11)
    phi = rng.standard_normal(shape).astype(F32)
    rec = _rec(L, [0.0, 0.0, 0.0], "fd")
    psi = [p.cpu().numpy() for p in baorec.compute_displacements(np.asfortranarray(phi), rec)]
    ref = O.fd_gradient_mesh(phi, L)
    for a in range(3):
        np.testing.assert_array_equal(psi[a], ref[a])


@pytest.mark.parametrize("field", ["disp", "sum"])
def test_fd_shifts_match_read_grad_cic(field):
    """:disp shifts are the reference's finite-difference read-out (FP64
    oracle) to FP32 rounding; :sum adds the RSD term of those shifts exactly
    as the FFT path does."""
    import baorec
    n, L = 48, F32(900.0)
    bm = [F32(100.0), F32(200.0), F32(300.0)]
    rng = np.random.default_rng(5)
    phi = O.smooth(rng.standard_normal((n, n, n)).astype(F32), 25.0, [L] * 3)
    rec = _rec([L] * 3, bm, "fd")
    x, y, z, _ = uniform_box(20000, L, seed=6)
    x, y, z = (x + bm[0]).astype(F32), (y + bm[1]).astype(F32), (z + bm[2]).astype(F32)
    got = baorec.read_shifts(rec, x, y, z, np.asfortranarray(phi), field=field)
    ref = O.read_grad_cic(phi, x, y, z, [L] * 3, bm)
    if field == "sum":
        ref = O.read_shifts(tuple(r.astype(F32) for r in ref), x, y, z, 0.8, field="sum")
    scale = max(float(np.abs(r).max()) for r in ref)
    for a in range(3):
        err = float(np.abs(got[a].astype(np.float64) - ref[a]).max())
        assert err < 2e-6 * scale, (a, err, scale)


def test_fd_matches_fft_on_smooth_field():
    """On a smooth field the central-difference gradient approaches the
    spectral one: relative difference ~ (k cell)^2 / 6 for the dominant
    mode (k cell = 0.2 here); switching back restores the FFT result."""
    import baorec
    n, L = 64, 1000.0
    g = (np.arange(n) + 0.5) * L / n
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    k = 2 * np.pi * 2 / L
    phi = (np.sin(k * X + 0.3) * np.cos(k * Y) + 0.5 * np.sin(k * Z + 1.0)).astype(F32)
    rec_fft = _rec([L] * 3, [0.0] * 3, "fft")
    rec_fd = _rec([L] * 3, [0.0] * 3, "fd")
    x, y, z, _ = uniform_box(5000, F32(L), seed=2)
    s_fft = baorec.read_shifts(rec_fft, x, y, z, np.asfortranarray(phi), field="disp")
    s_fd = baorec.read_shifts(rec_fd, x, y, z, np.asfortranarray(phi), field="disp")
    kc = k * L / n
    for a in range(3):
        rel = np.linalg.norm(s_fd[a] - s_fft[a]) / np.linalg.norm(s_fft[a])
        assert rel < 0.5 * kc ** 2, (a, rel)
        assert rel > 0.05 * kc ** 2          # the two gradients are different operators
    rec_fd.gradient = "fft"
    s_back = baorec.read_shifts(rec_fd, x, y, z, np.asfortranarray(phi), field="disp")
    for a in range(3):
        np.testing.assert_array_equal(s_back[a], s_fft[a])


def test_fd_rejected_for_iterative():
    from baorec import _lib
    cfg = _lib.default_config()
    cfg.method = _lib.ITERATIVE
    ctx = _lib.Context(cfg)
    with pytest.raises(_lib.BaorecError):
        ctx.call("baorec_set_gradient", 1)
    with pytest.raises(_lib.BaorecError):
        ctx.call("baorec_set_gradient", 7)
