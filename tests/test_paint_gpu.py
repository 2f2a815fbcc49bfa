"""Paint parity: the CUDA CIC/TSC paint against the oracle's restatement of
src/mas.jl.  Cell indices and counts are integers and must match bit for bit;
the mesh is an FP32 sum in a different order, compared with a tolerance."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, uniform_box

pytestmark = pytest.mark.gpu

# FP32 accumulation in a different order: per-cell relative tolerance
MESH_RTOL = 2e-5


@pytest.mark.parametrize("n,npart", [(16, 5000), (32, 50000), (24, 20000)])
def test_cell_bins_bit_exact(n, npart):
    import baorec
    L = F32(1000.0)
    x, y, z, w = uniform_box(npart, L, seed=n)
    # put some particles exactly on the upper boundary and on cell edges
    x[:10] = L
    y[10:20] = F32(0.0)
    z[20:30] = F32(L / n * 3)
    bs, bm = [L] * 3, [0.0] * 3
    keys, counts = baorec.cell_bins(x, y, z, bs, bm, (n, n, n), wrap=True)
    *_, okey = O.cell_keys(x, y, z, bs, bm, (n, n, n), wrap=True)
    np.testing.assert_array_equal(keys.astype(np.int64), okey)
    ocounts = O.cell_counts(x, y, z, bs, bm, (n, n, n), wrap=True)
    np.testing.assert_array_equal(counts.astype(np.int64), ocounts)
    assert counts.sum() == npart


@pytest.mark.parametrize("binned", [True, False])
@pytest.mark.parametrize("wrap", [True, False])
def test_cic_matches_oracle(wrap, binned):
    import baorec
    n, npart = 32, 40000
    L = F32(500.0)
    bmin = (F32(-10.0), F32(5.0), F32(0.0))
    x, y, z, w = uniform_box(npart, L * F32(0.9), seed=3, bmin=(0, 0, 0))
    x = (x + bmin[0] + F32(1)).astype(F32)
    y = (y + bmin[1] + F32(1)).astype(F32)
    z = (z + bmin[2] + F32(1)).astype(F32)
    bs = [L] * 3
    rho = baorec.zeros_mesh((n, n, n), device=False)
    gx, gy, gz = x.copy(), y.copy(), z.copy()
    baorec.cic_(rho, gx, gy, gz, w, bs, bmin, wrap=wrap, binned=binned)
    orho = np.zeros((n, n, n), F32)
    orho, opos = O.cic(orho, x, y, z, w, bs, bmin, wrap=wrap)
    np.testing.assert_allclose(rho, orho, rtol=MESH_RTOL, atol=1e-5 * float(np.abs(orho).max()))
    # mass conservation
    assert abs(float(rho.sum(dtype=np.float64)) - float(w.sum(dtype=np.float64))) < 1e-4 * float(w.sum())


def test_cic_wrap_mutates_positions_like_reference():
    import baorec
    n = 16
    L = F32(100.0)
    x = np.array([150.0, 50.0, 100.0, 99.999], F32)   # > L wraps, == L does not
    y = np.array([10.0, 120.0, 0.0, 5.0], F32)
    z = np.array([1.0, 2.0, 101.0, 3.0], F32)
    w = np.ones(4, F32)
    rho = baorec.zeros_mesh((n, n, n), device=False)
    gx, gy, gz = x.copy(), y.copy(), z.copy()
    baorec.cic_(rho, gx, gy, gz, w, [L] * 3, [0.0] * 3, wrap=True)
    _, (ox, oy, oz) = O.cic(np.zeros((n, n, n), F32), x, y, z, w, [L] * 3, [0.0] * 3, wrap=True)
    np.testing.assert_array_equal(gx, ox)
    np.testing.assert_array_equal(gy, oy)
    np.testing.assert_array_equal(gz, oz)
    assert gx[0] == F32(50.0) and gx[2] == F32(100.0)


def test_cic_out_of_bounds_raises_bounds_error():
    import baorec
    n = 8
    rho = baorec.zeros_mesh((n, n, n), device=False)
    x = np.array([10.0, -5.0], F32)
    y = np.array([10.0, 10.0], F32)
    z = np.array([10.0, 10.0], F32)
    with pytest.raises(IndexError):
        baorec.cic_(rho, x, y, z, np.ones(2, F32), [100.0] * 3, [0.0] * 3, wrap=True)
    with pytest.raises(IndexError):
        O.cic(np.zeros((n, n, n), F32), x, y, z, np.ones(2, F32), [100.0] * 3, [0.0] * 3, wrap=True)
    # without wrapping a particle in the last cell writes past the mesh
    x = np.array([99.0], F32)
    with pytest.raises(IndexError):
        baorec.cic_(rho, x, y[:1], z[:1], np.ones(1, F32), [100.0] * 3, [0.0] * 3, wrap=False)


def test_cic_empty_input():
    import baorec
    rho = baorec.zeros_mesh((8, 8, 8), device=False)
    e = np.zeros(0, F32)
    baorec.cic_(rho, e, e, e, e, [100.0] * 3, [0.0] * 3)
    assert not rho.any()


def test_cic_device_arrays():
    import torch
    import baorec
    n, npart = 32, 30000
    L = F32(1000.0)
    x, y, z, w = uniform_box(npart, L, seed=9)
    t = [torch.from_numpy(a.copy()).cuda() for a in (x, y, z, w)]
    rho = baorec.zeros_mesh((n, n, n))
    baorec.cic_(rho, *t, [L] * 3, [0.0] * 3)
    orho, _ = O.cic(np.zeros((n, n, n), F32), x, y, z, w, [L] * 3, [0.0] * 3)
    np.testing.assert_allclose(rho.cpu().numpy(), orho, rtol=MESH_RTOL, atol=1e-5 * float(orho.max()))


@pytest.mark.parametrize("shape", [(36, 30, 32), (30, 32, 28), (4, 8, 8)])
def test_cic_vector_and_scalar_reductions(shape):
    """x rows of a multiple of 4 cells take the 16-byte vector reductions
    (pairs inside an aligned group of four), others the scalar ones; every
    x residue is hit, including the pair that wraps from n-1 to 0."""
    import baorec
    npart = 60000
    L = [F32(300.0), F32(250.0), F32(200.0)]
    rng = np.random.default_rng(sum(shape))
    x, y, z = [(rng.random(npart) * float(L[a])).astype(F32) for a in range(3)]
    for p, l in zip((x, y, z), L):
        p[p >= l] = F32(0.0)
    w = (0.5 + rng.random(npart)).astype(F32)
    rho = baorec.zeros_mesh(shape, device=False)
    baorec.cic_(rho, x.copy(), y.copy(), z.copy(), w, L, [0.0] * 3, wrap=True, binned=False)
    orho, _ = O.cic(np.zeros(shape, F32), x, y, z, w, L, [0.0] * 3, wrap=True)
    np.testing.assert_allclose(rho, orho, rtol=MESH_RTOL, atol=1e-5 * float(orho.max()))


@pytest.mark.parametrize("binned", [True, False])
@pytest.mark.parametrize("wrap", [True, False])
def test_tsc_matches_oracle(wrap, binned):
    import baorec
    n, npart = 32, 30000
    L = F32(800.0)
    x, y, z, w = uniform_box(npart, L * F32(0.8), seed=5)
    x, y, z = [(a + F32(80)).astype(F32) for a in (x, y, z)]
    rho = baorec.zeros_mesh((n, n, n), device=False)
    baorec.tsc_(rho, x.copy(), y.copy(), z.copy(), w, [L] * 3, [0.0] * 3, wrap=wrap, binned=binned)
    orho, _ = O.tsc(np.zeros((n, n, n), F32), x, y, z, w, [L] * 3, [0.0] * 3, wrap=wrap)
    np.testing.assert_allclose(rho, orho, rtol=MESH_RTOL, atol=1e-5 * float(orho.max()))
    assert abs(float(rho.sum(dtype=np.float64)) - float(w.sum(dtype=np.float64))) < 1e-4 * float(w.sum())


@pytest.mark.parametrize("mas,wrap", [("cic", True), ("cic", False), ("tsc", True), ("tsc", False)])
def test_deterministic_paint_matches_oracle_and_repeats_bit_for_bit(mas, wrap):
    """The tile counting sort + fixed-point paint: the oracle's mesh within the
    paint tolerance, the atomic paint's within FP32 rounding, and the same
    bits on a second run (the atomic paint's sums depend on thread order)."""
    import baorec
    n, npart = 32, 60000
    L = F32(600.0)
    x, y, z, w = uniform_box(npart, L * F32(0.8), seed=11)
    x, y, z = [(a + F32(40)).astype(F32) for a in (x, y, z)]
    w = (w * F32(0.5) + F32(0.75)).astype(F32)
    bs, bm = [L] * 3, [0.0] * 3
    paint = baorec.cic_ if mas == "cic" else baorec.tsc_
    runs = []
    for _ in range(2):
        rho = baorec.zeros_mesh((n, n, n), device=False)
        paint(rho, x.copy(), y.copy(), z.copy(), w, bs, bm, wrap=wrap, deterministic=True)
        runs.append(np.array(rho))
    np.testing.assert_array_equal(runs[0].view(np.uint32), runs[1].view(np.uint32))
    fast = baorec.zeros_mesh((n, n, n), device=False)
    paint(fast, x.copy(), y.copy(), z.copy(), w, bs, bm, wrap=wrap)
    np.testing.assert_allclose(runs[0], fast, rtol=1e-5, atol=1e-6 * float(np.abs(fast).max()))
    ofn = O.cic if mas == "cic" else O.tsc
    orho, _ = ofn(np.zeros((n, n, n), F32), x.copy(), y.copy(), z.copy(), w, bs, bm, wrap=wrap)
    np.testing.assert_allclose(runs[0], orho, rtol=MESH_RTOL, atol=1e-5 * float(np.abs(orho).max()))


def test_deterministic_paint_wraps_across_the_periodic_edge():
    """Particles in the last cell of every axis (their upper CIC neighbour and
    TSC node wrap to cell 0) land where the atomic paint puts them."""
    import baorec
    n = 16
    L = F32(160.0)
    rng = np.random.default_rng(4)
    x = (L - rng.random(3000, dtype=np.float32) * F32(10)).astype(F32)
    y = (L - rng.random(3000, dtype=np.float32) * F32(10)).astype(F32)
    z = (rng.random(3000, dtype=np.float32) * L).astype(F32)
    w = np.ones(3000, F32)
    for paint in (baorec.cic_, baorec.tsc_):
        a = baorec.zeros_mesh((n, n, n), device=False)
        b = baorec.zeros_mesh((n, n, n), device=False)
        paint(a, x.copy(), y.copy(), z.copy(), w, [L] * 3, [0.0] * 3, wrap=True, deterministic=True)
        paint(b, x.copy(), y.copy(), z.copy(), w, [L] * 3, [0.0] * 3, wrap=True)
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-5)
        assert abs(float(np.sum(a, dtype=np.float64)) - 3000.0) < 1e-2


@pytest.mark.parametrize("mas", ["cic", "tsc"])
@pytest.mark.parametrize("shape,wrap", [((40, 24, 72), True), ((40, 24, 72), False), ((18, 33, 16), True),
                                        ((256, 256, 272), True)])
def test_binned_paint_partial_tiles_edges_and_accumulation(mas, shape, wrap):
    """The binned paint (tile counting sort, shared-memory tiles) against the
    oracle: meshes that are not multiples of the 16-cell tile (partial last
    tiles), one whose 16-cell tiles exceed the shared histogram (32-cell
    tiles), particles on tile boundaries, on the last cell of every axis (their
    upper weights wrap to cell 0) and on the upper box edge; the paint adds to
    the mesh it is given, as cic! does."""
    import baorec
    npart = 120000 if np.prod(shape) < 1e6 else 200000
    L = [F32(10.0 * s) for s in shape]
    rng = np.random.default_rng(sum(shape) + (7 if wrap else 0))
    lo = 0.0 if wrap else 25.0   # TSC / CIC weights stay inside the mesh without wrapping
    x, y, z = [(lo + rng.random(npart) * (float(L[a]) - 2 * lo)).astype(F32) for a in range(3)]
    # tile boundaries (cells 15/16, 31/32), the last cell, the upper edge
    k = npart // 8
    x[:k] = (F32(10.0) * rng.choice([15.5, 16.0, 31.99, 32.0], k)).astype(F32)
    if wrap:
        y[k:2 * k] = (L[1] - F32(10.0) * rng.random(k, dtype=np.float32)).astype(F32)
        z[2 * k:2 * k + 50] = L[2]
    w = (0.25 + rng.random(npart)).astype(F32)
    paint, ofn = (baorec.cic_, O.cic) if mas == "cic" else (baorec.tsc_, O.tsc)
    base = (rng.random(shape) - 0.5).astype(F32)
    rho = baorec.zeros_mesh(shape, device=False)
    rho[...] = base
    paint(rho, x.copy(), y.copy(), z.copy(), w, L, [0.0] * 3, wrap=wrap, binned=True)
    orho, _ = ofn(np.zeros(shape, F32), x.copy(), y.copy(), z.copy(), w, L, [0.0] * 3, wrap=wrap)
    got = np.asarray(rho, np.float64) - base
    np.testing.assert_allclose(got, orho, rtol=MESH_RTOL, atol=1e-5 * float(np.abs(orho).max()))
    assert abs(float(got.sum()) - float(w.sum(dtype=np.float64))) < 1e-4 * float(w.sum())


def test_binned_paint_out_of_bounds_raises_and_matches_atomic():
    """Without wrapping, a particle whose weights leave the mesh is the
    reference's BoundsError (IndexError) in both FP32 paints; the binned and
    atomic meshes of a valid catalogue agree to FP32 rounding."""
    import baorec
    n = 32
    L = F32(320.0)
    x, y, z, w = uniform_box(50000, L * F32(0.9), seed=13)
    x, y, z = [(a + F32(10)).astype(F32) for a in (x, y, z)]
    meshes = []
    for binned in (True, False):
        rho = baorec.zeros_mesh((n, n, n), device=False)
        baorec.cic_(rho, x.copy(), y.copy(), z.copy(), w, [L] * 3, [0.0] * 3, wrap=False, binned=binned)
        meshes.append(np.array(rho))
    np.testing.assert_allclose(meshes[0], meshes[1], rtol=1e-5, atol=1e-6 * float(np.abs(meshes[1]).max()))
    bad = x.copy()
    bad[7] = L - F32(1.0)   # last cell: its upper CIC weight would leave the mesh
    for binned in (True, False):
        with pytest.raises(IndexError):
            baorec.cic_(baorec.zeros_mesh((n, n, n), device=False), bad, y.copy(), z.copy(), w, [L] * 3,
                        [0.0] * 3, wrap=False, binned=binned)
