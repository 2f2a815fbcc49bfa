"""The oracle against the known-answer fixtures of tests/golden (exact
fractions and closed forms, made by tests/golden/make_golden.py) and its own
invariants.  CPU only."""
import os

import numpy as np
import pytest

import baorec_oracle as O

KAT = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kat.npz"))
F32 = np.float32


def test_cic_single_particles_exact():
    n = int(KAT["cic_n"])
    pos, w, box = KAT["cic_pos"], KAT["cic_w"], KAT["cic_box"]
    rho, _ = O.cic(np.zeros((n, n, n), F32), pos[:, 0], pos[:, 1], pos[:, 2], w, box, [0, 0, 0], wrap=True)
    # dyadic positions on a power-of-two cell: every FP32 operation is exact
    np.testing.assert_array_equal(rho.astype(np.float64), KAT["cic_mesh"])


def test_cic_mass_conservation_and_counts():
    rng = np.random.default_rng(0)
    n, L = 16, F32(100.0)
    x, y, z = (rng.random(5000).astype(F32) * L for _ in range(3))
    w = rng.random(5000).astype(F32)
    rho, _ = O.cic(np.zeros((n, n, n), np.float64), x, y, z, w, [L] * 3, [0, 0, 0])
    assert abs(rho.sum() - w.astype(np.float64).sum()) < 1e-9
    c = O.cell_counts(x, y, z, [L] * 3, [0, 0, 0], (n, n, n))
    assert c.sum() == 5000 and c.min() >= 0


def test_tsc_mass_conservation():
    rng = np.random.default_rng(1)
    n, L = 16, 100.0
    x, y, z = (rng.random(3000) * L for _ in range(3))
    w = np.ones(3000)
    rho, _ = O.tsc(np.zeros((n, n, n)), x, y, z, w, [L] * 3, [0, 0, 0])
    assert abs(rho.sum() - 3000.0) < 1e-9


def test_smooth_plane_wave():
    a = KAT["sm_in"]
    out = O.smooth(a.astype(np.float64), float(KAT["sm_R"]), [float(KAT["sm_L"])] * 3)
    np.testing.assert_allclose(out, KAT["sm_out"], atol=1e-12)


def test_restriction_and_prolongation_of_cosines():
    np.testing.assert_allclose(O.reduce(KAT["rs_fine"]), KAT["rs_coarse"], atol=1e-12)
    np.testing.assert_allclose(O.prolong(KAT["pr_coarse"], KAT["pr_fine"].shape), KAT["pr_fine"], atol=1e-12)


def test_read_cic_trilinear_exact():
    f = KAT["rd_field"]
    p = KAT["rd_pos"]
    L = float(KAT["rd_L"])
    out = O.read_cic(f.astype(np.float64), p[:, 0], p[:, 1], p[:, 2], [L] * 3, [0, 0, 0])
    np.testing.assert_allclose(out, KAT["rd_vals"], atol=1e-12)


def test_k_axes():
    n, L = int(KAT["kv_n"]), float(KAT["kv_L"])
    k = O.k_vec((n, n, n), [L] * 3, np.float64)
    np.testing.assert_allclose(k[0], KAT["kv_x"], rtol=1e-12)
    np.testing.assert_allclose(k[1], KAT["kv_y"], rtol=1e-12)


def test_setup_box_matches_reference_formula():
    x = np.array([1.0, 5.0, -2.0], F32)
    y = np.array([10.0, 0.0, 3.0], F32)
    z = np.array([0.5, 0.25, 7.0], F32)
    bs, bm = O.setup_box(x, y, z, 4.0)
    np.testing.assert_array_equal(bm, np.array([-4.0, -2.0, -1.75], F32))
    assert bs[0] == bs[1] == bs[2] == F32(14.0)


def test_iterate_global_los_plane_wave_closed_form():
    # δ = cos(k z), LOS = z: δ_k/k² · k_z² = δ_k, so one step gives δ_s - β/(1+β) δ
    n, L, beta = 16, 160.0, 0.4
    z = np.arange(n) * L / n
    d = np.broadcast_to(np.cos(2 * np.pi * 2 * z / L)[None, None, :], (n, n, n)).astype(np.float64)
    k = O.k_vec((n, n, n), [L] * 3, np.float64)
    out = O.iterate(d.copy(), d.copy(), k, 1, beta, los=(0.0, 0.0, 1.0))
    np.testing.assert_allclose(out, d * (1 - beta / (1 + beta)), atol=1e-12)


def test_operator_annihilates_constants_and_reduces_to_laplacian():
    n, L = 16, 160.0
    coef = O.stencil_coefficients((n, n, n), [L] * 3, [0.0] * 3, 0.0, los=(0.0, 0.0, 1.0), dtype=np.float64)
    ones = np.ones((n, n, n))
    np.testing.assert_allclose(O.apply_operator(ones, coef, False), 0.0, atol=1e-12)
    # β = 0: A = -∇² (7-point): A cos(kx) = (2 - 2cos kh)/h² cos(kx)
    x = np.arange(n) * L / n
    v = np.broadcast_to(np.cos(2 * np.pi * 3 * x / L)[:, None, None], (n, n, n))
    h = L / n
    np.testing.assert_allclose(O.apply_operator(v.copy(), coef, False),
                               (2 - 2 * np.cos(2 * np.pi * 3 / n)) / h ** 2 * v, atol=1e-10)


def test_convergent_solver_reaches_tolerance_in_fp64():
    rng = np.random.default_rng(2)
    n, L = 16, 400.0
    f = O.smooth(rng.standard_normal((n, n, n)), 40.0, [L] * 3)
    v, hist, alpha = O.solve_mg(f, np.array([L] * 3), np.array([-50.0, 20.0, 30.0]), 0.4, rtol=1e-10,
                                max_cycles=30)
    assert hist[-1] <= 1e-10
    assert all(b < a for a, b in zip(hist[1:], hist[2:]))


def test_fp32_oracle_close_to_fp64():
    rng = np.random.default_rng(3)
    n, L = 16, 300.0
    f = O.smooth(rng.standard_normal((n, n, n)), 30.0, [L] * 3)
    a = O.fmg(f.astype(F32), [L] * 3, [10.0, 20.0, 30.0], F32(0.4), F32(0.4), 5, 6)
    b = O.fmg(f, [L] * 3, [10.0, 20.0, 30.0], 0.4, 0.4, 5, 6)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-4
