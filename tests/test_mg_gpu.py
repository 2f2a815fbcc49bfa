"""Multigrid parity: primitives and the reference FMG schedule against the
oracle's restatement of src/multigrid.jl, and the residual-driven solver
against an FP64 evaluation of the residual of the same discrete operator."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, rel_l2, small_lightcone

pytestmark = pytest.mark.gpu


def _problem(n=32, seed=0, local=True):
    m = small_lightcone(n_data=30000, rand_factor=5, n_grid=n, seed=seed)
    bs, bm = O.setup_box(m.rx, m.ry, m.rz, 25.0 * 256 / n)
    f = O.setup_overdensity_randoms(np.zeros((n, n, n), F32), 2.0, 15.0, bs, bm, m.x, m.y, m.z, m.w,
                                    m.rx, m.ry, m.rz, m.rw)
    return f, bs, bm


def _recon(bs, bm, los=None, **kw):
    import baorec
    return baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm, los=los, **kw)


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0]])
def test_residual_and_jacobi_match_oracle(los):
    import baorec
    f, bs, bm = _problem()
    rec = _recon(bs, bm, los)
    rng = np.random.default_rng(1)
    v = O.smooth(rng.standard_normal(f.shape).astype(F32), 40.0, bs) * F32(100.0)
    r = baorec.zeros_mesh(f.shape, device=False)
    baorec.residual_(r, np.asfortranarray(v), np.asfortranarray(f), rec)
    ro = O.residual(v, f, bs, bm, rec.beta, los=los)
    assert rel_l2(r, ro) < 1e-4
    g = np.asfortranarray(v.copy())
    baorec.jacobi_(g, np.asfortranarray(f), rec, 3)
    jo = O.jacobi(v.copy(), f, bs, bm, rec.beta, 0.4, 3, los=los)
    assert rel_l2(g, jo) < 1e-6


def test_reduce_prolong_match_oracle():
    import baorec
    f, bs, bm = _problem(n=32)
    rec = _recon(bs, bm)
    c = baorec.zeros_mesh((16, 16, 16), device=False)
    baorec.reduce_(c, np.asfortranarray(f), rec, top_shape=f.shape)
    co = O.reduce(f)
    assert rel_l2(c, co) < 1e-6
    fine = baorec.zeros_mesh(f.shape, device=False)
    baorec.prolong_(fine, np.asfortranarray(co), rec, top_shape=f.shape)
    np.testing.assert_allclose(fine, O.prolong(co, f.shape), rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0]])
def test_fmg_reference_schedule_matches_oracle(los):
    import baorec
    f, bs, bm = _problem(n=32)
    rec = _recon(bs, bm, los)
    phi = baorec.fmg(np.asfortranarray(f), baorec.zeros_mesh(f.shape, device=False), rec)
    po = O.fmg(f, bs, bm, rec.beta, F32(0.4), 5, 6, los=los)
    # a long FP32 iteration: compare the potential and its gradient
    assert rel_l2(phi, po) < 1e-3
    g = O.gradient_meshes(np.asarray(phi, F32), bs)
    go = O.gradient_meshes(po, bs)
    assert max(rel_l2(g[a], go[a]) for a in range(3)) < 1e-3


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0]])
def test_convergent_solve_reaches_rtol_in_fp64(los):
    import baorec
    f, bs, bm = _problem(n=32, seed=3)
    rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40)
    phi = baorec.zeros_mesh(f.shape, device=False)
    st = baorec.solve_(phi, np.asfortranarray(f), rec)
    assert st["rel_residual"] <= 1e-6 and st["cycles"] <= 20
    # FP64 residual of the FP32 solution with the same coefficients (FP32 values, FP64 arithmetic)
    coef = O.coefs_f64(O.stencil_coefficients(f.shape, bs, bm, rec.beta, los, F32))
    r = (f.astype(np.float64) - st["alpha"]) - O.apply_operator(np.asarray(phi, np.float64), coef, los is None)
    fn = np.linalg.norm(f.astype(np.float64) - st["alpha"])
    assert np.linalg.norm(r) / fn < 2e-6


def test_convergent_solution_matches_fp64_oracle_gradient():
    import baorec
    f, bs, bm = _problem(n=32, seed=5)
    rec = _recon(bs, bm, None, mg_mode="convergent", rtol=1e-7, max_cycles=40)
    phi = baorec.zeros_mesh(f.shape, device=False)
    baorec.solve_(phi, np.asfortranarray(f), rec)
    v64, hist, _ = O.solve_mg(f.astype(np.float64), bs.astype(np.float64), bm.astype(np.float64), rec.beta,
                           los=None, rtol=1e-10, max_cycles=40)
    g = O.gradient_meshes(np.asarray(phi, np.float64), bs.astype(np.float64))
    go = O.gradient_meshes(v64, bs.astype(np.float64))
    err = max(rel_l2(g[a], go[a]) for a in range(3))
    assert err < 1e-5, err


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0], [0.6, 0.0, 0.8]])
def test_spectral_start_reaches_same_solution_with_fewer_cycles(los):
    """FFT-preconditioned corrections first (mean line of sight), then
    V-cycles: the same FP64-checked residual, fewer V-cycles than the zero
    start, the same gradient."""
    import baorec
    f, bs, bm = _problem(n=64, seed=7)
    ff = np.asfortranarray(f)
    out = {}
    for start in ("zero", "spectral"):
        rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40, start=start)
        phi = baorec.zeros_mesh(f.shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        coef = O.coefs_f64(O.stencil_coefficients(f.shape, bs, bm, rec.beta, los, F32))
        r = (f.astype(np.float64) - st["alpha"]) - O.apply_operator(np.asarray(phi, np.float64), coef, los is None)
        assert np.linalg.norm(r) / np.linalg.norm(f.astype(np.float64) - st["alpha"]) < 2e-6
        out[start] = (st, O.gradient_meshes(np.asarray(phi, np.float64), bs.astype(np.float64)))
    s0, g0 = out["zero"]
    s1, g1 = out["spectral"]
    assert s0["spectral_steps"] == 0 and s1["spectral_steps"] >= 1
    print("zero", s0, "spectral", s1)
    assert s1["cycles"] < s0["cycles"], (s0, s1)
    if los is not None:
        # one line of sight: the FFT inverse is exact, no V-cycle is needed
        assert s1["cycles"] == 0, s1
    assert max(rel_l2(g1[a], g0[a]) for a in range(3)) < 2e-5


def test_fft_start_callback_and_kernel_forms_agree():
    """The preconditioner multiply as a cuFFT LTO load callback (when cuFFT
    can build that plan) and as a separate kernel: same converged solution;
    a request cuFFT cannot honour falls back to the kernel and says why."""
    import baorec
    f, bs, bm = _problem(n=64, seed=7)
    ff = np.asfortranarray(f)
    grads, states = [], []
    for enable in (1, 0):
        rec = _recon(bs, bm, None, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, f.shape)
        ctx.call("baorec_set_fft_callbacks", enable)
        phi = baorec.zeros_mesh(f.shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        states.append(ctx.fft_callbacks())
        grads.append(O.gradient_meshes(np.asarray(phi, np.float64), bs.astype(np.float64)))
    print(states)
    assert states[0]["state"] in (1, -1)
    if states[0]["state"] == -1:
        assert "unavailable" in states[0]["note"]
    assert states[1]["state"] == -1
    assert max(rel_l2(grads[0][a], grads[1][a]) for a in range(3)) < 2e-5


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0]])
def test_streaming_and_tiled_residual_kernels_agree(los):
    """The z-marching, cp.async-pipelined residual kernels and the tiled ones:
    the same solve history within rounding and the same converged gradient."""
    import baorec
    f, bs, bm = _problem(n=64, seed=12)
    ff = np.asfortranarray(f)
    out = []
    for form in (0, 1):
        rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, f.shape)
        ctx.call("baorec_set_tune_stream", form)
        phi = baorec.zeros_mesh(f.shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        hist = ctx.solve_history()
        out.append((st, hist, O.gradient_meshes(np.asarray(phi, np.float64), bs.astype(np.float64))))
    (s0, h0, g0), (s1, h1, g1) = out
    assert [k for _, k in h0] == [k for _, k in h1]
    for (r0, _), (r1, _) in zip(h0, h1):
        assert abs(r0 - r1) <= 1e-3 * r0 + 1e-9
    assert max(rel_l2(g1[a], g0[a]) for a in range(3)) < 1e-5


@pytest.mark.parametrize("start", ["zero", "spectral"])
def test_zero_start_first_residual_is_exact_one(start):
    """A zero solution's residual is f - α with α = mean f: the solve records
    relative residual 1 without a stencil pass, and still converges to the
    FP64-checked 1e-6 of the oracle operator."""
    import baorec
    f, bs, bm = _problem(n=64, seed=3)
    rec = _recon(bs, bm, None, mg_mode="convergent", rtol=1e-6, max_cycles=40, start=start)
    ctx = baorec.setup_fft_(rec, f.shape)
    phi = baorec.zeros_mesh(f.shape, device=False)
    st = baorec.solve_(phi, np.asfortranarray(f), rec)
    hist = ctx.solve_history()
    assert hist[0][0] == 1.0 and st["rel_residual_initial"] == 1.0
    assert st["rel_residual"] <= 1e-6
    coef = O.coefs_f64(O.stencil_coefficients(f.shape, bs, bm, rec.beta, None, F32))
    r = (f.astype(np.float64) - st["alpha"]) - O.apply_operator(np.asarray(phi, np.float64), coef, True)
    assert np.linalg.norm(r) / np.linalg.norm(f.astype(np.float64) - st["alpha"]) < 2e-6


@pytest.mark.parametrize("los", [None, [0.0, 0.0, 1.0], [0.6, 0.0, 0.8]])
def test_pair_and_single_cell_running_residuals_agree(los):
    """The FP32 running residual on 32x16x16 tiles with two z-adjacent cells
    per thread (packed FP32x2, plane-pair window) and with one cell per
    thread: the same residual of the FFT start to FP32 rounding, the same
    solve history and the same converged gradient."""
    import ctypes as C
    import baorec
    f, bs, bm = _problem(n=64, seed=12)
    ff = np.asfortranarray(f)
    out = []
    for pairs in (0, 1):
        rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, f.shape)
        ctx.call("baorec_set_tune", 8, (C.c_int32 * 16)(*([1] * 16)))   # 16x16 tiles wherever they fit
        ctx.call("baorec_set_tune_stream", 0)
        ctx.call("baorec_set_tune_pairs", pairs)
        assert ctx.lib.baorec_tune_pairs(ctx.h) == pairs
        phi = baorec.zeros_mesh(f.shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        out.append((st, ctx.solve_history(), O.gradient_meshes(np.asarray(phi, np.float64), bs.astype(np.float64))))
    (s0, h0, g0), (s1, h1, g1) = out
    print(h0, h1)
    assert [k for _, k in h0] == [k for _, k in h1]
    for (r0, _), (r1, _) in zip(h0, h1):
        assert abs(r0 - r1) <= 1e-3 * r0 + 1e-9
    assert max(rel_l2(g1[a], g0[a]) for a in range(3)) < 1e-5


@pytest.mark.parametrize("los", [None, [0.0, 0.6, 0.8]])
def test_z_pass_preconditioner_matches_3d_transforms(los):
    """The FFT preconditioner as batched xy transforms around the fused z pass
    (four-step 256-point transforms, the k-space multiply between them) and as
    3-D transforms with a separate multiply: the same residual of the FFT
    start, the same solve history and the same converged potential, on a
    non-cubic mesh with 256 z planes."""
    import torch
    import baorec
    from baorec import guess
    shape = (32, 64, 256)
    bs = np.array([400.0, 800.0, 3200.0], F32)
    bm = np.array([600.0, -400.0, -1600.0], F32)
    rng = np.random.default_rng(21)
    f = O.smooth(rng.standard_normal(shape).astype(F32), 40.0, bs)
    f = (f - f.mean(dtype=np.float64)).astype(F32)
    ff = np.asfortranarray(f)
    fd = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).cuda()
    rels, outs = [], []
    for zp in (0, 1, 2):
        rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, shape)
        ctx.call("baorec_set_tune_zpass", zp)
        assert ctx.lib.baorec_tune_zpass(ctx.h) == zp
        rels.append(guess.start_residual(ctx, fd.data_ptr(), "spectral"))
        phi = baorec.zeros_mesh(shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        outs.append((st, ctx.solve_history(), np.asarray(phi, np.float64)))
    print(rels, [h for _, h, _ in outs])
    (s0, h0, p0) = outs[0]
    for rel, (s1, h1, p1) in zip(rels[1:], outs[1:]):
        assert abs(rels[0] - rel) <= 1e-4 * rels[0] + 2e-6
        assert [k for _, k in h0] == [k for _, k in h1]
        assert rel_l2(p1 - p1.mean(), p0 - p0.mean()) < 1e-5


def test_cycle_cap_returns_not_converged_with_the_last_iterate():
    """At the V-cycle cap the solve returns BAOREC_ERR_NOT_CONVERGED, φ holds
    the last iterate (its FP64 residual is the reported one), and the plain
    method continued from that iterate reaches the tolerance."""
    import baorec
    from baorec import _lib
    f, bs, bm = _problem(n=32, seed=3)
    ff = np.asfortranarray(f)
    rec = _recon(bs, bm, None, mg_mode="convergent", rtol=1e-6, max_cycles=1, start="zero")
    phi = baorec.zeros_mesh(f.shape, device=False)
    with pytest.raises(_lib.NotConverged):
        baorec.solve_(phi, ff, rec)
    st = rec.solve_stats
    assert st["status"] == _lib.ERR_NOT_CONVERGED
    assert st["cycles"] == 1 and st["rel_residual"] > 1e-6
    coef = O.coefs_f64(O.stencil_coefficients(f.shape, bs, bm, rec.beta, None, F32))
    r = (f.astype(np.float64) - st["alpha"]) - O.apply_operator(np.asarray(phi, np.float64), coef, True)
    rel = np.linalg.norm(r - r.mean()) / np.linalg.norm(f.astype(np.float64) - st["alpha"])
    assert abs(rel - st["rel_residual"]) <= 0.05 * st["rel_residual"], (rel, st)
    # the fallback: more V-cycles from the capped iterate
    rec2 = _recon(bs, bm, None, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="zero")
    phi2 = baorec.zeros_mesh(f.shape, device=False)
    st2 = baorec.solve_(phi2, ff, rec2, phi0=np.asfortranarray(phi))
    assert st2["rel_residual"] <= 1e-6
    assert st2["rel_residual_initial"] <= 1.05 * st["rel_residual"]


@pytest.mark.parametrize("shape,los", [((64, 64, 64), None), ((32, 48, 96), [0.0, 0.6, 0.8]), ((64, 32, 48), None),
                                       ((128, 64, 64), None), ((64, 64, 32), [0.0, 0.0, 1.0])])
def test_streamed_pair_running_residual_is_bit_identical(shape, los):
    """Every packed form of the running residual does the pair kernel's
    arithmetic cell for cell: the window streamed through a ring of plane
    pairs (16- and 32-plane blocks; the 32-plane form falls back to 16 where
    n3 is not a multiple of 32), and the TMA-staged form with x-adjacent pairs
    (32- and 16-plane columns; it falls back to the pair kernel where n1 is
    not a multiple of 64, n2 not of 16 or n3 not of the column length), and
    the pair kernel on 32x8x16 tiles of 256 threads.  The FFT start's
    residual, the solve history and the solution are the same bits."""
    import ctypes as C
    import torch
    import baorec
    from baorec import guess
    bs = np.array([10.0 * s for s in shape], F32) * F32(9.0)
    bm = np.array([300.0, -200.0, 150.0], F32)
    rng = np.random.default_rng(31)
    f = O.smooth(rng.standard_normal(shape).astype(F32), 40.0, bs)
    f = (f - f.mean(dtype=np.float64)).astype(F32)
    ff = np.asfortranarray(f)
    fd = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).cuda()
    out = []
    for pairs in (1, 2, 3, 4, 5, 6):
        rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, shape)
        ctx.call("baorec_set_tune", 8, (C.c_int32 * 16)(*([1] * 16)))
        ctx.call("baorec_set_tune_stream", 0)
        ctx.call("baorec_set_tune_pairs", pairs)
        assert ctx.lib.baorec_tune_pairs(ctx.h) == pairs
        rel = guess.start_residual(ctx, fd.data_ptr(), "spectral")
        phi = baorec.zeros_mesh(shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        out.append((rel, ctx.solve_history(), np.asarray(phi).copy()))
    for rel, hist, phi in out[1:]:
        assert rel == out[0][0]
        assert hist == out[0][1]
        np.testing.assert_array_equal(phi, out[0][2])


@pytest.mark.parametrize("los", [None, [0.0, 0.6, 0.8]])
def test_accurate_residual_block_shapes_agree(los):
    """The accurate residual (double-float solution update) on 512-thread
    blocks and on 256-thread blocks of 32x8x8 and 32x8x16 tiles: the same
    per-cell arithmetic, so the solve takes the same steps and reaches the
    same solution; only the per-block partial sums of the residual norm are
    grouped differently: FP32 sums within a block's threads, so the history
    agrees to FP32 rounding of those sums (1e-5 relative)."""
    import ctypes as C
    import baorec
    f, bs, bm = _problem(n=64, seed=21)
    ff = np.asfortranarray(f)
    out = []
    for acc in (0, 1, 2):
        rec = _recon(bs, bm, los, mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, f.shape)
        ctx.call("baorec_set_tune", 8, (C.c_int32 * 16)(*([1] * 16)))
        ctx.call("baorec_set_tune_stream", 0)
        ctx.call("baorec_set_tune_acc", acc)
        assert ctx.lib.baorec_tune_acc(ctx.h) == acc
        phi = baorec.zeros_mesh(f.shape, device=False)
        st = baorec.solve_(phi, ff, rec)
        assert st["rel_residual"] <= 1e-6
        out.append((ctx.solve_history(), np.asarray(phi, np.float64).copy()))
    h0, p0 = out[0]
    for h, p in out[1:]:
        assert [k for _, k in h] == [k for _, k in h0]
        for (r, _), (r0, _) in zip(h, h0):
            assert abs(r - r0) <= 1e-5 * r0
        assert np.max(np.abs(p - p0)) <= 1e-5 * np.max(np.abs(p0))
    assert ctx.status("baorec_set_tune_acc", 3) == baorec._lib.ERR_ARG
