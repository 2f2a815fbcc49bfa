"""Catalog I/O on the host (no context, no GPU): the ASCII reader against the
oracle's exact decimal-to-FP32 rounding, the threaded path on a file large
enough to be split, the error reports, and the .npy layout npzwrite gives
hcat(x, y, z)."""
import numpy as np
import pytest

import catalog_oracle as CO

TRICKY = ["0.1", "-2.5", "1e-45", "7.006e-46", "1.00000005960464477539062501", "1.000000059604644775390625",
          "1.0000001788139343", "3.4028235e38", "16777217", "123456.789", "-0.0", "1.5E+03", "+4.25",
          "0.000012345678", "9.999999e-39", "2.350988561514728583455765982071533026645717985517980855365926236850006129930346077117064851336181163787841796875e-38"]


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_reader_matches_exact_rounding(tmp_path):
    from baorec import catalog
    rng = np.random.default_rng(0)
    lines = ["# ra dec d z nz", "header line to skip"]
    toks = list(TRICKY)
    for v in rng.normal(size=200) * 10.0 ** rng.integers(-8, 9, 200):
        toks.append(rng.choice(["%.6f", "%.9e", "%.18e", "%g", "%.3f"]) % v)
    rows = []
    for i in range(0, len(toks) - 4, 5):
        rows.append("  ".join(toks[i:i + 5]) + ("\t" if i % 3 else ""))
        if i % 7 == 0:
            rows.append("")
        if i % 11 == 0:
            rows.append("   # a comment")
    text = "\n".join([lines[1], lines[0]] + rows) + "\n"
    path = _write(tmp_path, "cat.txt", text)
    got = catalog.read_ascii(path, [0, 2, 4], skip=1, comment="#")
    ref = CO.read_ascii(text, [0, 2, 4], skip=1, comment="#")
    for g, r in zip(got, ref):
        assert g.dtype == np.float32
        np.testing.assert_array_equal(g.view(np.uint32), r.view(np.uint32))


def test_reader_threads_on_large_file(tmp_path):
    """~8 MB: split across the host threads; %.9g of an FP32 value reads back
    to the same bits, rows stay in file order."""
    from baorec import catalog
    rng = np.random.default_rng(1)
    n = 120_000
    cols = [rng.uniform(-1e3, 1e3, n).astype(np.float32), rng.lognormal(0, 3, n).astype(np.float32),
            (rng.normal(size=n) * 1e-5).astype(np.float32), np.arange(n, dtype=np.float32)]
    text = "\n".join("%.9g %.9g %.9g %.9g" % (a, b, c, d) for a, b, c, d in zip(*cols)) + "\n"
    path = _write(tmp_path, "big.txt", text)
    got = catalog.read_ascii(path, [3, 0, 1, 2])
    for g, r in zip(got, [cols[3], cols[0], cols[1], cols[2]]):
        np.testing.assert_array_equal(g.view(np.uint32), r.view(np.uint32))


def test_reader_errors(tmp_path):
    import ctypes as C
    from baorec import _lib, catalog
    p = _write(tmp_path, "short.txt", "1 2 3\n4 5 6\n7 8\n")
    with pytest.raises(_lib.BaorecError, match="line 3"):
        catalog.read_ascii(p, [0, 2])
    p = _write(tmp_path, "bad.txt", "1 2\n3 4.5.6\n")
    with pytest.raises(_lib.BaorecError, match="line 2"):
        catalog.read_ascii(p, [1])
    with pytest.raises(_lib.BaorecError, match="cannot open"):
        catalog.read_ascii(str(tmp_path / "missing.txt"), [0])
    # more rows than the output room
    p = _write(tmp_path, "ok.txt", "1\n2\n3\n")
    lib = _lib.load()
    cols = (C.c_int32 * 1)(0)
    buf = np.zeros(2, np.float32)
    outs = (C.c_void_p * 1)(buf.ctypes.data)
    nr = C.c_int64()
    st = lib.baorec_read_ascii(None, p.encode(), cols, 1, 0, 0, outs, 2, C.byref(nr), _lib.HOST)
    assert st == _lib.ERR_TOO_LARGE and nr.value == 3


def test_empty_file_reads_no_rows(tmp_path):
    from baorec import catalog
    p = _write(tmp_path, "empty.txt", "# only a comment\n\n")
    got = catalog.read_ascii(p, [0, 1])
    assert [len(g) for g in got] == [0, 0]


def test_write_npy_layout(tmp_path):
    from baorec import catalog
    rng = np.random.default_rng(2)
    x, y, z = (rng.normal(size=1001).astype(np.float32) for _ in range(3))
    p = str(tmp_path / "pos.npy")
    catalog.write_npy(p, [x, y, z])
    a = np.load(p)
    assert a.shape == (1001, 3) and a.dtype == np.float32 and a.flags.f_contiguous
    np.testing.assert_array_equal(a[:, 0], x)
    np.testing.assert_array_equal(a[:, 2], z)
    raw = open(p, "rb").read()
    hl = raw[8] | (raw[9] << 8)
    assert (10 + hl) % 64 == 0 and raw[10 + hl - 1:10 + hl] == b"\n"
    catalog.write_npy(str(tmp_path / "empty.npy"), [np.zeros(0, np.float32)] * 2)
    assert np.load(str(tmp_path / "empty.npy")).shape == (0, 2)
