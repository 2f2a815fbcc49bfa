"""Learned initial guess: the device network (tensor-core forward, backward
data and weight-gradient kernels) against the CPU oracle of the same network
with BF16 rounding, and its use as the start of the residual-driven solve."""
import numpy as np
import pytest

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


@pytest.mark.parametrize("seed", [0, 1])
def test_network_forward_and_gradients_match_oracle(seed):
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
    loss = C.c_double()
    ctx.call("baorec_guess_eval", fd.data_ptr(), td.data_ptr(), out.data_ptr(), grads.ctypes.data, C.byref(loss))
    lo, oo, go = GO.loss_and_grads(p, feats, target, n, bf16=True)
    _, o64, g64 = GO.loss_and_grads(p, feats, target, n, bf16=False)
    o = out.cpu().numpy().reshape(n, n, n)
    assert rel_l2(o, oo) < 1e-2, rel_l2(o, oo)
    assert abs(loss.value - lo) / lo < 1e-2
    lay, total = GO.layout()
    for l, (wo, shape, bo, nb) in enumerate(lay):
        for a, b in ((wo, wo + int(np.prod(shape))), (bo, bo + nb)):
            noise = rel_l2(go[a:b], g64[a:b])
            assert rel_l2(grads[a:b], go[a:b]) < 0.7 * noise + 0.02, (l, rel_l2(grads[a:b], go[a:b]), noise)
            assert rel_l2(grads[a:b], g64[a:b]) < 1.5 * noise + 0.02, (l, rel_l2(grads[a:b], g64[a:b]), noise)
