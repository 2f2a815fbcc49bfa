"""tcgen05 convolution of the learned guess (TMA-staged BF16 operands, TMEM
accumulators) against an FP64 convolution of the same BF16 inputs, against
the mma.sync kernel, and inside the network (forward and gradients)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TC_SHAPES = [(8, 16), (16, 16), (32, 32), (32, 16), (16, 32), (32, 64), (64, 32)]


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


def _bf16(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16)


def _sample_voxels(n, rng, count=6000):
    """Random voxels plus whole boundary rows (x = 0 and n-1 ends, y and z faces)."""
    z = rng.integers(0, n, count)
    y = rng.integers(0, n, count)
    x = rng.integers(0, n, count)
    xs = np.arange(n)
    rows = [(0, 0), (n - 1, n - 1), (0, n - 1), (n // 2, 0), (n - 1, n // 3)]
    for zz, yy in rows:
        z = np.concatenate([z, np.full(n, zz)])
        y = np.concatenate([y, np.full(n, yy)])
        x = np.concatenate([x, xs])
    return z, y, x


def _conv_ref(xf, w, bias, add, relu, z, y, x):
    """FP64 3x3x3 zero-padded convolution at the voxels (z, y, x); xf is the
    (n, n, n, cin) input as FP32 copies of its BF16 entries (exact)."""
    n = xf.shape[0]
    cols = []
    for t in range(27):
        zz, yy, xx = z + t // 9 - 1, y + (t // 3) % 3 - 1, x + t % 3 - 1
        ok = (zz >= 0) & (zz < n) & (yy >= 0) & (yy < n) & (xx >= 0) & (xx < n)
        v = xf[np.clip(zz, 0, n - 1), np.clip(yy, 0, n - 1), np.clip(xx, 0, n - 1)].astype(np.float64)
        v[~ok] = 0.0
        cols.append(v)
    patches = np.stack(cols, axis=1)                      # (S, 27, cin)
    out = np.einsum("stc,tco->so", patches, w)
    if bias is not None:
        out += bias[None, :]
    if add is not None:
        out += add[z, y, x].astype(np.float64)
    if relu:
        out = np.maximum(out, 0.0)
    return out


@pytest.mark.parametrize("n", [128, 64])
@pytest.mark.parametrize("cin,cout", TC_SHAPES)
def test_conv3_tcgen05_matches_fp64_and_mma(cin, cout, n):
    """Every covered shape at n = 128 (one full tile per row) and n = 64 (one
    half-used tile per row: the upper 64 slots read the TMA zero fill and are
    not stored), both slab loaders: the tcgen05 output equals the FP64
    convolution of the same BF16 operands to BF16 output rounding, and the
    mma.sync kernel's output to within one BF16 step (the two differ only in
    the FP32 summation order)."""
    import torch
    from baorec import guess
    rng = np.random.default_rng(cin * 100 + cout + n)
    ctx = _ctx(n)
    xb = _bf16(rng.normal(size=(n, n, n, cin)))
    wq = _bf16(rng.normal(scale=1.0 / np.sqrt(27 * cin), size=(27, cin, cout))).to(torch.float32)
    bias = torch.from_numpy(rng.normal(scale=0.1, size=cout).astype(np.float32))
    xd, wd, bd = xb.cuda(), wq.cuda(), bias.cuda()
    y_mma = guess.conv3(ctx, xd, wd, bd, relu=False, path="mma").float().cpu().numpy()
    z, y, x = _sample_voxels(n, rng)
    ref = _conv_ref(xb.float().numpy(), wq.double().numpy(), bias.double().numpy(), None, False, z, y, x)
    outs = {}
    for path in ("tcgen05", "tcgen05_cpasync"):
        y_tc = guess.conv3(ctx, xd, wd, bd, relu=False, path=path).float().cpu().numpy()
        got = y_tc[z, y, x]
        # BF16 rounding of the output (2^-8 relative) plus FP32 accumulation
        tol = 2.0 ** -8 * np.abs(ref) + 1e-4
        assert np.all(np.abs(got - ref) <= tol), (path, float(np.max(np.abs(got - ref) - tol)))
        d = np.abs(y_tc - y_mma)
        # one BF16 step, plus the FP32 reassociation error of a 27*cin-term
        # sum that cancels to a small output (the tensor core adds partial
        # accumulators in another order than the mma.sync kernel)
        step = 2.0 ** -7 * np.maximum(np.abs(y_tc), np.abs(y_mma)) + 1e-5
        assert np.all(d <= step), (path, float(np.max(d - step)))
        assert np.mean(d == 0) > 0.98, (path, np.mean(d == 0))
        outs[path] = y_tc
    # the two loaders fill identical slabs: identical results
    assert np.array_equal(outs["tcgen05"], outs["tcgen05_cpasync"])


def test_conv3_tcgen05_addend_relu_n256():
    """The epilogue with an addend and ReLU, n = 256 (two 128-voxel segments
    per row), against the FP64 reference."""
    import torch
    from baorec import guess
    n, cin, cout = 256, 16, 16
    rng = np.random.default_rng(7)
    ctx = _ctx(n)
    xb = _bf16(rng.normal(size=(n, n, n, cin)))
    ab = _bf16(rng.normal(scale=0.5, size=(n, n, n, cout)))
    wq = _bf16(rng.normal(scale=1.0 / np.sqrt(27 * cin), size=(27, cin, cout))).to(torch.float32)
    bias = torch.from_numpy(rng.normal(scale=0.1, size=cout).astype(np.float32))
    y_tc = guess.conv3(ctx, xb.cuda(), wq.cuda(), bias.cuda(), add=ab.cuda(), relu=True, path="tcgen05")
    y_tc = y_tc.float().cpu().numpy()
    z, y, x = _sample_voxels(n, rng)
    ref = _conv_ref(xb.float().numpy(), wq.double().numpy(), bias.double().numpy(), ab.float().numpy(), True,
                    z, y, x)
    got = y_tc[z, y, x]
    tol = 2.0 ** -8 * np.abs(ref) + 1e-4
    assert np.all(np.abs(got - ref) <= tol), float(np.max(np.abs(got - ref) - tol))
    assert np.mean(got == 0) > 0.2   # ReLU was applied


def test_conv3_tcgen05_rejects_uncovered():
    """Shapes or grids without a tcgen05 kernel are an argument error, not a
    silent fallback."""
    import torch
    from baorec import _lib, guess
    ctx = _ctx(96)
    x = torch.zeros((96, 96, 96, 16), dtype=torch.bfloat16, device="cuda")
    w = torch.zeros((27, 16, 16), device="cuda")
    with pytest.raises(_lib.BaorecError):
        guess.conv3(ctx, x, w, path="tcgen05")       # n = 96: neither a multiple of 128 nor 64
    ctx = _ctx(128)
    x = torch.zeros((128, 128, 128, 64), dtype=torch.bfloat16, device="cuda")
    w = torch.zeros((27, 64, 64), device="cuda")
    with pytest.raises(_lib.BaorecError):
        guess.conv3(ctx, x, w, path="tcgen05")       # 64 -> 64 channels: mma.sync only


@pytest.mark.parametrize("n", [256, 128])
def test_network_tcgen05_matches_mma_forward_and_gradients(n):
    """The whole network with the trained weights at n = 256 and at n = 128
    (the size it runs at on the first restriction of a 256^3 mesh): output
    and parameter gradients with the tcgen05 layers on and off agree to the
    BF16 noise of the activations; the forward ran the eight covered layers
    (four at n^3, four at (n/2)^3; the 64->64 layers at (n/4)^3 have no
    tcgen05 kernel) on tcgen05."""
    import torch
    from baorec import guess
    ctx = _ctx(n)
    p = guess.load_params(guess.os.path.join(guess.WEIGHTS_DIR, "guess_lightcone.npy"))
    guess.set_params(ctx, p)
    rng = np.random.default_rng(3)
    fd = torch.from_numpy(rng.normal(size=(n, n, n, 8)).astype(np.float32)).cuda()
    td = torch.from_numpy(rng.normal(size=(n, n, n)).astype(np.float32)).cuda()
    res = {}
    for tc in (True, False):
        guess.set_conv_path(ctx, tc)
        out = torch.empty(n ** 3, device="cuda")
        grads = np.zeros(guess.num_params(), np.float32)
        lval = C.c_double()
        ctx.call("baorec_guess_eval", fd.data_ptr(), td.data_ptr(), out.data_ptr(), grads.ctypes.data, C.byref(lval), 0)
        res[tc] = (out.cpu().numpy(), grads, lval.value, guess.tc_layers(ctx))
    o1, g1, l1, k1 = res[True]
    o0, g0, l0, k0 = res[False]
    assert k1 == 8 and k0 == 0, (k1, k0)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    assert rel(o1, o0) < 1e-2, rel(o1, o0)
    assert abs(l1 - l0) / l0 < 1e-3
    assert rel(g1, g0) < 2e-2, rel(g1, g0)


def test_expired_waits_return_a_status_and_leave_the_context_usable():
    """The bounded waits of the tcgen05 convolution: with the slab loader held
    back and every pipeline wait limited to 20 µs, the waits expire, the
    kernel records the timeout (no trap, no fault), every role stops, the
    block waits for its weight copy and frees its TMEM, and the call returns a
    status.  The context then runs a normal convolution that equals the
    mma.sync kernel's, and a second expiry behaves the same."""
    import torch
    from baorec import _lib, guess
    n = 128
    ctx = _ctx(n)
    rng = np.random.default_rng(5)
    for _ in range(2):
        st = ctx.status("baorec_guess_conv3_held_back", 16, 16, n, 20_000)
        assert st == _lib.ERR_CUDA
        assert "timed out" in ctx.lib.baorec_last_error(ctx.h).decode()
        x = _bf16(rng.normal(size=(n, n, n, 16))).cuda()
        w = torch.from_numpy(rng.normal(scale=0.1, size=(27, 16, 16)).astype(np.float32)).cuda()
        y_tc = guess.conv3(ctx, x, w, relu=False, path="tcgen05")
        y_ms = guess.conv3(ctx, x, w, relu=False, path="mma")
        a, b = y_tc.float().cpu().numpy(), y_ms.float().cpu().numpy()
        assert np.max(np.abs(a - b)) <= 2e-2 * np.max(np.abs(b)), np.max(np.abs(a - b))
    # shapes without a tcgen05 kernel are refused before any launch
    assert ctx.status("baorec_guess_conv3_held_back", 16, 16, 96, 20_000) == _lib.ERR_ARG
