"""Read-out parity: given the same mesh, the fused CUDA read-out reproduces the
oracle's restatement of read_cic!/read_shifts/reconstructed_positions bit for
bit (both evaluate the reference's FP32 expression order without FMA)."""
import numpy as np
import pytest

import baorec_oracle as O
from _util import F32, small_lightcone, uniform_box

pytestmark = pytest.mark.gpu


def _field(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, n, n)).astype(F32)


@pytest.mark.parametrize("n", [16, 32])
def test_read_cic_bit_exact(n):
    import baorec
    L = F32(300.0)
    bm = [F32(-50.0), F32(10.0), F32(0.0)]
    fld = _field(n, n)
    x, y, z, _ = uniform_box(20000, L, seed=n + 1)
    x, y, z = (x + bm[0]).astype(F32), (y + bm[1]).astype(F32), (z + bm[2]).astype(F32)
    out = np.empty(len(x), F32)
    baorec.read_cic_(out, np.asfortranarray(fld), x, y, z, [L] * 3, bm)
    ref = O.read_cic(fld, x, y, z, [L] * 3, bm)
    np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("los", [None, (0.0, 0.0, 1.0)])
@pytest.mark.parametrize("field", ["disp", "rsd", "sum"])
def test_shifts_and_positions_bit_exact(los, field):
    import baorec
    n, L = 32, F32(900.0)
    bm = [F32(100.0), F32(200.0), F32(300.0)]
    rng = np.random.default_rng(3)
    fld = O.smooth(rng.standard_normal((n, n, n)).astype(F32), 30.0, [L] * 3)
    rec = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=bm,
                                los=None if los is None else list(los))
    x, y, z, _ = uniform_box(10000, L, seed=4)
    x, y, z = (x + bm[0]).astype(F32), (y + bm[1]).astype(F32), (z + bm[2]).astype(F32)
    # the displacement meshes come from the GPU; the read-out arithmetic is compared exactly
    psi = [p.cpu().numpy() for p in baorec.compute_displacements(np.asfortranarray(fld), rec)]
    disp = tuple(O.read_cic(p, x, y, z, [L] * 3, bm) for p in psi)
    ref = O.read_shifts(disp, x, y, z, 0.8, los=los, field=field)
    got = baorec.read_shifts(rec, x, y, z, np.asfortranarray(fld), field=field)
    for a in range(3):
        np.testing.assert_array_equal(got[a], ref[a])
    pos = baorec.reconstructed_positions(rec, x, y, z, np.asfortranarray(fld), field=field)
    rpos = O.reconstructed_positions(ref, x, y, z)
    for a in range(3):
        np.testing.assert_array_equal(pos[a], rpos[a])


@pytest.mark.parametrize("device", [False, True])
def test_positions2_equals_two_calls(device):
    """The fused two-field read-out gives exactly the two single calls."""
    import torch
    import baorec
    n, L = 32, F32(900.0)
    bm = [F32(100.0), F32(200.0), F32(300.0)]
    rng = np.random.default_rng(9)
    fld = O.smooth(rng.standard_normal((n, n, n)).astype(F32), 30.0, [L] * 3)
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=bm)
    x, y, z, _ = uniform_box(10000, L, seed=10)
    x, y, z = (x + bm[0]).astype(F32), (y + bm[1]).astype(F32), (z + bm[2]).astype(F32)
    if device:
        x, y, z = (torch.from_numpy(a).cuda() for a in (x, y, z))
    a, b = baorec.reconstructed_positions2(rec, x, y, z, np.asfortranarray(fld), fields=("sum", "disp"))
    ra = baorec.reconstructed_positions(rec, x, y, z, np.asfortranarray(fld), field="sum")
    rb = baorec.reconstructed_positions(rec, x, y, z, np.asfortranarray(fld), field="disp")
    conv = (lambda t: t.cpu().numpy()) if device else (lambda t: t)
    for u, v in zip(a + b, ra + rb):
        np.testing.assert_array_equal(conv(u), conv(v))


def test_chunked_host_readout_equals_device():
    """Host arrays above two chunks take the pipelined read-out (copy-in,
    read-out and copy-out of consecutive chunks overlap on three streams):
    outputs equal the device-array call bit for bit, ragged last chunk
    included."""
    import torch
    import baorec
    n, L = 32, F32(900.0)
    bm = [F32(100.0), F32(200.0), F32(300.0)]
    rng = np.random.default_rng(11)
    fld = O.smooth(rng.standard_normal((n, n, n)).astype(F32), 30.0, [L] * 3)
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=bm)
    npart = 3 * (1 << 20) + 12345
    x, y, z, _ = uniform_box(npart, L, seed=12)
    x, y, z = (x + bm[0]).astype(F32), (y + bm[1]).astype(F32), (z + bm[2]).astype(F32)
    xd, yd, zd = (torch.from_numpy(a).cuda() for a in (x, y, z))
    a, b = baorec.reconstructed_positions2(rec, x, y, z, np.asfortranarray(fld), fields=("sum", "disp"))
    ad, bd = baorec.reconstructed_positions2(rec, xd, yd, zd, np.asfortranarray(fld), fields=("sum", "disp"))
    for u, v in zip(a + b, ad + bd):
        np.testing.assert_array_equal(u, v.cpu().numpy())
    s = baorec.read_shifts(rec, x, y, z, np.asfortranarray(fld), field="rsd")
    sd = baorec.read_shifts(rec, xd, yd, zd, np.asfortranarray(fld), field="rsd")
    for u, v in zip(s, sd):
        np.testing.assert_array_equal(u, v.cpu().numpy())


def test_page_locked_host_arrays_used_in_place():
    """Page-locked (pinned) host arrays are read and written by the kernels in
    place over the host link, with no staging: the reconstruction from pinned
    catalogs (deterministic paint) and the read-out into pinned outputs, above
    two pipeline chunks, equal the device-array calls bit for bit."""
    import ctypes as C
    import torch
    import baorec
    from baorec import _lib
    m = small_lightcone(n_data=20000, rand_factor=5, n_grid=32, seed=4)
    n = 32
    bs, bm = O.setup_box(m.rx, m.ry, m.rz, 200.0)
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm,
                                mg_mode="convergent", rtol=1e-6, start="spectral")
    ctx = baorec.setup_fft_(rec, (n, n, n))
    cats = [m.x, m.y, m.z, m.w, m.rx, m.ry, m.rz, m.rw]
    pin = [torch.from_numpy(np.ascontiguousarray(a, dtype=F32)).pin_memory() for a in cats]
    dev = [t.cuda() for t in pin]
    npart = 2 * (1 << 20) + 777
    rng = np.random.default_rng(8)
    q = [(bm[a] + rng.random(npart) * bs[a]).astype(F32) for a in range(3)]
    qpin = [torch.from_numpy(a).pin_memory() for a in q]
    qdev = [t.cuda() for t in qpin]
    res = []
    for cat, pos, loc in ((dev, qdev, "cuda"), (pin, qpin, "pin")):
        flags = _lib.HOST if loc == "pin" else 0
        p = [t.data_ptr() for t in cat]
        ctx.call("baorec_reconstructed_potential", *p[:4], len(m.x), *p[4:], len(m.rx), flags | _lib.DETERMINISTIC)
        phi = torch.empty(n ** 3, device="cuda")
        ctx.call("baorec_get_result", C.c_void_p(phi.data_ptr()), 0)
        outs = [torch.empty(npart, device="cuda") if loc == "cuda" else torch.empty(npart).pin_memory()
                for _ in range(6)]
        o = [t.data_ptr() for t in outs]
        ctx.call("baorec_reconstructed_positions2", *[t.data_ptr() for t in pos], npart,
                 _lib.FIELD["sum"], *o[:3], _lib.FIELD["disp"], *o[3:], flags)
        torch.cuda.synchronize()
        res.append((phi.cpu().numpy(), [t.cpu().numpy() for t in outs]))
    (p0, o0), (p1, o1) = res
    np.testing.assert_array_equal(p0, p1)
    for u, v in zip(o0, o1):
        np.testing.assert_array_equal(u, v)
