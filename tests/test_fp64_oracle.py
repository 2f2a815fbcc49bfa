"""The FP64 accuracy judge (oracle/fp64_oracle.py) against the NumPy
restatement of src/multigrid.jl: the C operator equals
baorec_oracle.apply_operator with the same FP32 coefficients in FP64
arithmetic, and its FFT-preconditioned solution equals the V-cycle solution
of baorec_oracle.solve_mg.  CPU only."""
import numpy as np
import pytest

import baorec_oracle as O
import fp64_oracle as P
from _util import F32, small_lightcone

BETA = F32(F32(0.8) / F32(2.0))


def _rhs(n, seed):
    m = small_lightcone(n_data=30000, rand_factor=5, n_grid=n, seed=seed)
    bs, bm = O.setup_box(m.rx, m.ry, m.rz, 25.0 * 256 / n)
    f = O.setup_overdensity_randoms(np.zeros((n, n, n), F32), 2.0, 15.0, bs, bm, m.x, m.y, m.z, m.w,
                                    m.rx, m.ry, m.rz, m.rw)
    return f, bs, bm


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0], [0.6, 0.0, 0.8]])
def test_c_operator_equals_numpy_operator(los):
    shape = (16, 24, 32)
    bs = np.array([400.0, 600.0, 800.0], F32)
    bm = np.array([300.0, -200.0, 100.0], F32)
    v = np.random.default_rng(3).standard_normal(shape)
    got = P.Operator(shape, bs, bm, BETA, los).apply(v)
    coef = O.coefs_f64(O.stencil_coefficients(shape, bs, bm, BETA, los, F32))
    want = O.apply_operator(v, coef, los is None)
    # same FP32 coefficients, FP64 arithmetic: equal to the last bits
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0]])
def test_fp64_solution_equals_vcycle_solution(los):
    f, bs, bm = _rhs(32, 5)
    phi, alpha, hist = P.solve(f, bs, bm, BETA, los, rtol=1e-11)
    assert hist[-1] <= 1e-11
    # its own residual, recomputed with the NumPy operator
    coef = O.coefs_f64(O.stencil_coefficients(f.shape, bs, bm, BETA, los, F32))
    r = (f.astype(np.float64) - alpha) - O.apply_operator(np.asarray(phi), coef, los is None)
    assert np.linalg.norm(r) / np.linalg.norm(f.astype(np.float64) - alpha) <= 1e-11
    v64, _, alpha2 = O.solve_mg(f.astype(np.float64), bs.astype(np.float64), bm.astype(np.float64), BETA,
                                los=los, rtol=1e-11, max_cycles=60)
    assert abs(alpha - alpha2) <= 1e-8 * abs(alpha2)
    g1 = P.gradient_meshes(phi, bs.astype(np.float64))
    g2 = O.gradient_meshes(v64, bs.astype(np.float64))
    assert P.rel_l2_vector(g1, g2) < 1e-7


def test_fp64_gradient_equals_oracle_gradient():
    rng = np.random.default_rng(9)
    phi = rng.standard_normal((16, 16, 32))
    bs = np.array([300.0, 300.0, 600.0])
    g1 = P.gradient_meshes(phi, bs)
    g2 = O.gradient_meshes(phi, bs)
    assert P.rel_l2_vector(g1, g2) < 1e-14
