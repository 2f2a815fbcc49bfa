"""Catalog I/O with device arrays: the reader's device columns equal its host
columns; shifted positions written from device tensors (streamed through the
pinned staging blocks, several blocks per column) read back exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_read_equals_host(tmp_path):
    from baorec import catalog
    rng = np.random.default_rng(3)
    n = 50_000
    vals = rng.normal(size=(n, 5)).astype(np.float32)
    p = tmp_path / "cat.txt"
    p.write_text("\n".join(" ".join("%.9g" % v for v in row) for row in vals) + "\n")
    host = catalog.read_ascii(str(p), [0, 1, 3, 4])
    dev = catalog.read_ascii(str(p), [0, 1, 3, 4], device=True)
    for h, d in zip(host, dev):
        np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), h.view(np.uint32))


def test_write_npy_from_device(tmp_path):
    import torch
    from baorec import catalog
    n = 9_000_001                                  # > 2 staging blocks of 4 Mi floats per column
    cols = [torch.randn(n, device="cuda") for _ in range(3)]
    p = str(tmp_path / "rec.npy")
    catalog.write_npy(p, cols)
    a = np.load(p, mmap_mode="r")
    assert a.shape == (n, 3) and a.dtype == np.float32
    for k in range(3):
        np.testing.assert_array_equal(np.asarray(a[:, k]), cols[k].cpu().numpy())
