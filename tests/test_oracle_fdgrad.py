"""Oracle of the finite-difference read-out (src/mas.jl:388-466): its
per-particle formula equals the CIC read of the central-difference mesh,
and on a sinusoid it is the exact central difference at the nodes."""
import numpy as np

import baorec_oracle as O


def test_read_grad_cic_is_cic_of_difference_mesh():
    n, L, bm = 16, [300.0, 240.0, 360.0], [5.0, -3.0, 0.0]
    rng = np.random.default_rng(0)
    phi = rng.standard_normal((n, n, n))
    x, y, z = (rng.uniform(b, b + l, 2000) for b, l in zip(bm, L))
    g = O.read_grad_cic(phi, x, y, z, L, bm)
    mesh = O.fd_gradient_mesh(phi, L)
    r = [O.read_cic(m, x, y, z, L, bm) for m in mesh]
    for a in range(3):
        np.testing.assert_allclose(g[a], r[a], rtol=0, atol=1e-12)


def test_read_grad_cic_at_nodes_is_central_difference():
    n, L = 32, 640.0
    d = L / n
    k = 2 * np.pi * 3 / L
    xs = np.arange(n) * d
    phi = np.broadcast_to(np.sin(k * xs)[:, None, None], (n, n, n)).copy()
    x = xs + 0.0
    y = np.full(n, 7 * d)
    z = np.full(n, 11 * d)
    gx, gy, gz = O.read_grad_cic(phi, x, y, z, [L] * 3, [0.0] * 3)
    exact = (np.sin(k * (xs + d)) - np.sin(k * (xs - d))) / (2 * d)
    np.testing.assert_allclose(gx, exact, rtol=0, atol=1e-12)
    assert np.abs(gy).max() < 1e-12 and np.abs(gz).max() < 1e-12


def test_fd_gradient_mesh_fp32_wraps():
    phi = np.arange(4 * 5 * 6, dtype=np.float32).reshape(4, 5, 6)
    gx, gy, gz = O.fd_gradient_mesh(phi, [8.0, 10.0, 12.0])
    c2 = np.float32(np.float32(16.0) / np.float32(4))
    assert gx.dtype == np.float32
    assert gx[0, 0, 0] == np.float32((phi[1, 0, 0] - phi[3, 0, 0]) / c2)
    assert gx[3, 2, 1] == np.float32((phi[0, 2, 1] - phi[2, 2, 1]) / c2)
