"""Fused 2-D real transforms of 256 x 256 xy planes (xyfft.cu: packed
128-point row transforms and 256-point four-step column transforms on a
four-CTA cluster per plane, one kernel per direction) against cuFFT's batched
2-D transforms and the oracle,
through the three paths that use them on meshes of 256 z planes: smoothing,
the displacement spectra and the FFT preconditioner."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, rel_l2

pytestmark = pytest.mark.gpu

SHAPE = (256, 256, 256)
BS = [1500.0, 1500.0, 1500.0]


@pytest.mark.parametrize("xy", [0, 1])
def test_smooth_256_matches_oracle(xy):
    import baorec
    from baorec import recon
    a = np.random.default_rng(3).standard_normal(SHAPE).astype(F32)
    ctx = recon._prim_ctx(SHAPE, BS, [0.0, 0.0, 0.0], smoothing_radius=15.0)
    ctx.call("baorec_set_tune_xy", xy)
    assert ctx.lib.baorec_tune_xy(ctx.h) == xy
    g = np.asfortranarray(a.copy())
    baorec.smooth_(g, 15.0, BS)
    ctx.call("baorec_set_tune_xy", 1)
    o = O.smooth(a, 15.0, BS)
    assert rel_l2(g, o) < 2e-6


def test_displacement_256_fused_matches_cufft_and_oracle():
    import baorec
    fld = O.smooth(np.random.default_rng(4).standard_normal(SHAPE).astype(F32), 20.0, BS)
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=BS, box_min=[0.0] * 3)
    ctx = baorec.setup_fft_(rec, SHAPE)
    out = {}
    for xy in (0, 1):
        ctx.call("baorec_set_tune_xy", xy)
        psi = baorec.compute_displacements(np.asfortranarray(fld), rec)
        out[xy] = [p.cpu().numpy() for p in psi]
    ctx.call("baorec_set_tune_xy", 1)
    for a in range(3):
        assert rel_l2(out[1][a], out[0][a]) < 2e-6
    ref = O.gradient_meshes(fld, BS)
    for a in range(3):
        assert rel_l2(out[1][a], ref[a]) < 1e-5


@pytest.mark.parametrize("los", [None, [0.0, 0.6, 0.8]])
def test_preconditioner_256_fused_matches_cufft(los):
    """The FFT start's residual and the converged solve agree between the
    fused xy kernels and cuFFT's transforms."""
    import torch
    import baorec
    from baorec import guess
    f = O.smooth(np.random.default_rng(5).standard_normal(SHAPE).astype(F32), 30.0, BS)
    f = (f - f.mean(dtype=np.float64)).astype(F32)
    fd = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).cuda()
    bm = [400.0, -700.0, -750.0]
    rels, phis, hists = [], [], []
    for xy in (0, 1):
        rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=BS, box_min=bm, los=los,
                                    mg_mode="convergent", rtol=1e-6, max_cycles=40, start="spectral")
        ctx = baorec.setup_fft_(rec, SHAPE)
        ctx.call("baorec_set_tune_xy", xy)
        rels.append(guess.start_residual(ctx, fd.data_ptr(), "spectral"))
        phi = baorec.zeros_mesh(SHAPE, device=False)
        st = baorec.solve_(phi, np.asfortranarray(f), rec)
        assert st["rel_residual"] <= 1e-6
        hists.append([k for _, k in ctx.solve_history()])
        phis.append(np.asarray(phi, np.float64))
    print(rels, hists)
    if los is None:
        assert abs(rels[0] - rels[1]) <= 1e-4 * rels[0] + 2e-6
    else:
        # one line of sight: S⁻¹ is the operator's exact inverse, and both start
        # residuals sit at the FP32 rounding floor of A S⁻¹ f (different roundings)
        assert max(rels) < 1e-3
    assert hists[0] == hists[1]
    assert rel_l2(phis[1] - phis[1].mean(), phis[0] - phis[0].mean()) < 1e-5


def _mg_context(n):
    from baorec import _lib
    cfg = _lib.default_config()
    cfg.method = _lib.MULTIGRID
    cfg.mg_mode = _lib.MG_CONVERGENT
    for a, lo in enumerate((500.0, 300.0, 200.0)):
        cfg.n[a] = n
        cfg.box_size[a] = 2000.0 * n / 256
        cfg.box_min[a] = lo
    return _lib.Context(cfg)


def test_profile_hook_times_both_xy_transform_paths():
    """baorec_profile_kernel 8 / 9 time the batched xy transforms of the
    finest mesh by the current choice (cuFFT or the fused kernels) and report
    their algorithmic bytes: the real mesh plus the half spectrum."""
    import ctypes as C
    from baorec import _lib
    ctx = _mg_context(256)
    want = 4.0 * 256 ** 3 + 8.0 * 129 * 256 * 256
    for xy in (0, 1):
        ctx.call("baorec_set_tune_xy", xy)
        for which in (8, 9):
            avg, nbytes = C.c_float(), C.c_double()
            ctx.call("baorec_profile_kernel", which, 3, C.byref(avg), C.byref(nbytes))
            assert nbytes.value == want
            assert 0.0 < avg.value < 10.0


def test_profile_hook_rejects_meshes_without_batched_xy_transforms():
    import ctypes as C
    from baorec import _lib
    ctx = _mg_context(64)
    avg, nbytes = C.c_float(), C.c_double()
    with pytest.raises(_lib.BaorecError, match="xy") as e:
        ctx.call("baorec_profile_kernel", 8, 3, C.byref(avg), C.byref(nbytes))
    assert e.value.code == _lib.ERR_ARG
