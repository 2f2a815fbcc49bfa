"""Learned initial guess: the device network (tensor-core forward, backward
data and weight-gradient kernels) against the CPU oracle of the same network
with BF16 rounding, and its use as the start of the residual-driven solve."""
import numpy as np
import pytest

import baorec_oracle as O
import guess_oracle as GO
from _util import rel_l2

pytestmark = pytest.mark.gpu


def _ctx(n, box=1000.0, bmin=(500.0, 300.0, 200.0)):
    from baorec import _lib
    c = _lib.default_config()
    c.method = _lib.MULTIGRID
    for a in range(3):
        c.n[a] = n
        c.box_size[a] = box
        c.box_min[a] = bmin[a]
    c.mg_mode = _lib.MG_CONVERGENT
    return _lib.Context(c)


@pytest.mark.parametrize("seed,loss", [(0, "mse"), (1, "laplacian")])
def test_network_forward_and_gradients_match_oracle(seed, loss):
    """Forward output and every layer's weight and bias gradient against the
    oracle with the device's BF16 rounding points.  The tolerance of each
    gradient is set by the BF16 noise of that layer (the BF16 oracle against
    the exact FP64 one): a wrong kernel is off by O(1), rounding is not."""
    import ctypes as C
    import torch
    n = 32
    ctx = _ctx(n)
    rng = np.random.default_rng(seed)
    p32 = GO.init_params(seed, head_scale=0.3).astype(np.float32)   # kept alive across the call
    ctx.call("baorec_guess_set_params", p32.ctypes.data, p32.size)
    p = p32.astype(np.float64)
    feats = rng.normal(size=(n, n, n, 8)).astype(np.float32)
    target = rng.normal(size=(n, n, n)).astype(np.float32)
    fd = torch.from_numpy(feats).cuda()
    td = torch.from_numpy(target).cuda()
    out = torch.empty(n ** 3, device="cuda")
    grads = np.zeros(p.size, np.float32)
    lval = C.c_double()
    ctx.call("baorec_guess_eval", fd.data_ptr(), td.data_ptr(), out.data_ptr(), grads.ctypes.data, C.byref(lval),
             {"mse": 0, "laplacian": 1}[loss])
    lo, oo, go = GO.loss_and_grads(p, feats, target, n, bf16=True, loss=loss)
    _, o64, g64 = GO.loss_and_grads(p, feats, target, n, bf16=False, loss=loss)
    o = out.cpu().numpy().reshape(n, n, n)
    assert rel_l2(o, oo) < 1e-2, rel_l2(o, oo)
    assert abs(lval.value - lo) / lo < 1e-2
    lay, total = GO.layout()
    # errors relative to the block's gradient, floored at 1e-4 of the whole
    # gradient (the Laplacian loss makes the head bias gradient exactly zero)
    floor = 1e-4 * np.linalg.norm(g64)
    err = lambda x, y: float(np.linalg.norm(x - y) / max(np.linalg.norm(y), floor))
    for l, (wo, shape, bo, nb) in enumerate(lay):
        for a, b in ((wo, wo + int(np.prod(shape))), (bo, bo + nb)):
            noise = err(go[a:b], g64[a:b])
            assert err(grads[a:b], go[a:b]) < 0.7 * noise + 0.02, (l, err(grads[a:b], go[a:b]), noise)
            assert err(grads[a:b], g64[a:b]) < 1.5 * noise + 0.02, (l, err(grads[a:b], g64[a:b]), noise)


def test_trained_network_improves_the_fft_start_and_keeps_the_solution():
    """The committed parameters (trained on the device by baorec.train_guess)
    against the untrained network and the FFT start on unseen fields of the
    training distribution, and a learned-start solve against the FFT-start
    solve of the same field (same converged gradient)."""
    import torch
    import baorec
    from baorec import guess, train_guess
    # the committed parameters were trained on the 128^3 restriction of the 256^3 lightcone box
    ctx, cfg = train_guess.training_context(128, 128)
    guess.init(ctx, 3)
    untrained = train_guess.held_out(ctx, cfg, count=4)
    guess.set_params(ctx, guess.load_params(f"{guess.WEIGHTS_DIR}/guess_lightcone.npy"))
    trained = train_guess.held_out(ctx, cfg, count=4)
    r_un = np.mean([b / a for a, b in untrained])
    r_tr = np.mean([b / a for a, b in trained])
    print("learned / FFT start residual: untrained %.3f, trained %.3f" % (r_un, r_tr))
    # trained for 20k Adam steps (batch 4) at this geometry: about 0.37 of the FFT start's residual
    assert r_tr < 0.5 and r_tr < r_un
    # the learned start changes the path, not the answer
    n = 128
    f = torch.empty(n ** 3, device="cuda")
    phi = torch.empty(n ** 3, device="cuda")
    guess.sample(ctx, cfg, 20_000_000, f.data_ptr(), phi.data_ptr())
    bs, bm = ctx.box()
    fa = f.cpu().numpy().reshape(n, n, n)
    grads = {}
    for start in ("spectral", "learned"):
        rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm,
                                    mg_mode="convergent", rtol=1e-6, start=start,
                                    guess_params=guess.load_params(f"{guess.WEIGHTS_DIR}/guess_lightcone.npy")
                                    if start == "learned" else None)
        ph = baorec.zeros_mesh((n, n, n), device=False)
        st = baorec.solve_(ph, np.asfortranarray(fa.transpose(2, 1, 0)), rec)
        assert st["rel_residual"] <= 1e-6
        grads[start] = (st, O.gradient_meshes(np.asarray(ph, np.float64), np.asarray(bs, np.float64)))
    print("spectral", grads["spectral"][0], "learned", grads["learned"][0])
    g0, g1 = grads["spectral"][1], grads["learned"][1]
    assert max(rel_l2(g1[a], g0[a]) for a in range(3)) < 2e-5


def test_learned_start_on_the_restriction_of_the_lightcone_mesh():
    """guess_level 1 on the 256^3 lightcone mesh: the network runs on the
    128^3 restriction (full weighting in, trilinear prolongation out, the
    operators of src/multigrid.jl:398-453, 520-584), which is where the
    committed parameters were trained.  The parameters move to the child
    context and back, the learned start's residual is below the FFT start's,
    and the solve from it converges to the FFT start's solution."""
    import torch
    import baorec
    from baorec import _lib, guess, mocks
    W = guess.load_params(f"{guess.WEIGHTS_DIR}/guess_lightcone.npy")
    n = 256
    m = mocks.lightcone_mock(n_data=200_000, rand_factor=10, n_grid=n, seed=77)
    bs, bm = O.setup_box(m.rx, m.ry, m.rz, 25.0)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    X = [dev(a) for a in (m.x, m.y, m.z, m.w)]
    Rr = [dev(a) for a in (m.rx, m.ry, m.rz, m.rw)]
    recs = {}
    for start in ("spectral", "learned"):
        recs[start] = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm,
                                            mg_mode="convergent", rtol=1e-6, start=start,
                                            guess_params=W if start == "learned" else None, guess_level=1)
    ctx = baorec.setup_fft_(recs["learned"], (n,) * 3)
    assert ctx.lib.baorec_guess_level(ctx.h) == 1
    np.testing.assert_array_equal(guess.get_params(ctx), W)
    f = baorec.zeros_mesh((n,) * 3)
    baorec.setup_overdensity_(f, recs["spectral"], *X, *Rr)
    r_fft = guess.start_residual(ctx, f.data_ptr(), "spectral")
    r_l = guess.start_residual(ctx, f.data_ptr(), "learned")
    print("256^3 start residual: FFT %.4f, learned on the restriction %.4f (ratio %.3f)" % (r_fft, r_l, r_l / r_fft))
    # a perfect correction on the restriction would give about 0.77 (the prolonged correction leaves the
    # error's fine-scale part); the trained network gives about 0.83
    assert r_l < 0.9 * r_fft
    grads = {}
    for start, rec in recs.items():
        phi = baorec.zeros_mesh((n,) * 3)
        st = baorec.solve_(phi, f, rec)
        assert st["rel_residual"] <= 1e-6, st
        grads[start] = O.gradient_meshes(phi.cpu().numpy().astype(np.float64), bs.astype(np.float64))
    assert max(rel_l2(grads["learned"][a], grads["spectral"][a]) for a in range(3)) < 2e-5
    # back to level 0: the parameters move with the network
    ctx.call("baorec_guess_set_level", 0)
    assert ctx.lib.baorec_guess_level(ctx.h) == 0
    np.testing.assert_array_equal(guess.get_params(ctx), W)
    assert ctx.status("baorec_guess_set_level", 2) == _lib.ERR_ARG


def test_learned_start_is_the_fft_start_for_a_fixed_line_of_sight():
    """With one line of sight the FFT start is the exact inverse of the
    operator: the learned start equals it (no network correction) and both
    start at the residual the FFT's rounding leaves."""
    import torch
    import baorec
    from baorec import guess
    W = guess.load_params(f"{guess.WEIGHTS_DIR}/guess_lightcone.npy")
    n = 128
    rng = np.random.default_rng(4)
    bs = np.array([1500.0] * 3, np.float32)
    f = O.smooth(rng.standard_normal((n, n, n)).astype(np.float32), 30.0, bs)
    fd = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).cuda()
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=[0.0] * 3,
                                los=[0.0, 0.0, 1.0], mg_mode="convergent", rtol=1e-6, start="learned",
                                guess_params=W, guess_level=1)
    ctx = baorec.setup_fft_(rec, (n,) * 3)
    torch.cuda.synchronize()
    r_fft = guess.start_residual(ctx, fd.data_ptr(), "spectral")
    r_l = guess.start_residual(ctx, fd.data_ptr(), "learned")
    print("fixed line of sight: FFT start", r_fft, "learned", r_l)
    # the FFT start is the exact inverse here: what is left is FP32 rounding of the transforms
    assert r_l == r_fft and r_fft < 1e-4
