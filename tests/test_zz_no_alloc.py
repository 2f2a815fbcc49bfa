"""baorec_setup_box_noalloc: the bounding box for callers that cannot let the
library allocate device memory (a host whose pool allocator owns the device
memory budget, or a pipeline that cannot afford cudaMalloc's device-wide
synchronisation).  Its answer must equal the allocating entry point
baorec_setup_box and the oracle's setup_box (src/utils.jl:100-109) on the same
inputs, on consecutive calls that share the one fixed scratch array.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 16_777_216   # 1024 blocks x 256 threads x 64 particles


def _noalloc(lib, x, y, z, pad, stream=None):
    bs = (C.c_float * 3)()
    bm = (C.c_float * 3)()
    st = lib.baorec_setup_box_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
                                      x.numel(), C.c_float(pad), stream, bs, bm)
    return st, np.array(list(bs), np.float32), np.array(list(bm), np.float32)


def test_setup_box_noalloc_matches_allocating_entry_point():
    import torch
    import baorec
    import baorec_oracle as O
    from baorec import _lib
    lib = baorec.load_library()
    torch.cuda.set_device(0)
    side = torch.cuda.Stream()
    # consecutive calls with different inputs share the fixed scratch array:
    # sizes that fill part of the last block, fewer particles than one block,
    # a single particle, and one call on a stream of the caller's own
    cases = ((1_000_003, 1, 500.0, None), (3_000_000, 2, 25.0, None), (5_000, 3, 25.0, None),
             (1, 4, 10.0, None), (2_500_001, 5, 500.0, side))
    for n, seed, pad, stream in cases:
        g = torch.Generator(device="cuda").manual_seed(seed)
        x = torch.rand(n, device="cuda", generator=g) * 1500.0 - 200.0
        y = torch.rand(n, device="cuda", generator=g) * 900.0 + 10.0
        z = torch.rand(n, device="cuda", generator=g) * 1200.0
        torch.cuda.synchronize()
        st, bs, bm = _noalloc(lib, x, y, z, pad, None if stream is None else C.c_void_p(stream.cuda_stream))
        assert st == _lib.OK
        ebs, ebm = baorec.setup_box(x, y, z, pad)
        obs, obm = O.setup_box(x.cpu().numpy(), y.cpu().numpy(), z.cpu().numpy(), pad)
        # min/max and the FP32 box arithmetic are exact: tolerance zero
        np.testing.assert_array_equal(bs, ebs)
        np.testing.assert_array_equal(bm, ebm)
        np.testing.assert_array_equal(bs, obs)
        np.testing.assert_array_equal(bm, obm)


def test_setup_box_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    import baorec
    from baorec import _lib
    lib = baorec.load_library()
    x = torch.zeros(4, device="cuda")
    bs = (C.c_float * 3)()
    bm = (C.c_float * 3)()
    p = C.c_void_p(x.data_ptr())
    # the size check happens before any device access
    assert lib.baorec_setup_box_noalloc(p, p, p, MAX_PARTICLES + 1, C.c_float(1.0), None, bs, bm) == _lib.ERR_TOO_LARGE
    assert lib.baorec_setup_box_noalloc(p, p, p, 0, C.c_float(1.0), None, bs, bm) == _lib.ERR_ARG
    # host memory is refused before any launch: the kernels only read device memory
    h = np.zeros(4, np.float32)
    hp = C.c_void_p(h.ctypes.data)
    assert lib.baorec_setup_box_noalloc(hp, hp, hp, 4, C.c_float(1.0), None, bs, bm) == _lib.ERR_ARG
