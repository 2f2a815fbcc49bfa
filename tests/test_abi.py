"""The C-ABI library loads and exports every symbol include/baorec_gb300.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(baorec_[a-z0-9_]+)\s*\(", src, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("baorec_create", "baorec_run", "baorec_cic", "baorec_mg_fmg", "baorec_reconstructed_positions"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared but not exported"


def test_python_binding_covers_header(lib):
    from baorec import _lib
    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_config_defaults_match_reference(lib):
    from baorec import _lib
    c = _lib.default_config()
    # IterativeRecon / MultigridRecon defaults (src/recon.jl:10, 26-28) and setup_overdensity! ran_min
    assert c.n_iter == 3
    assert abs(c.jacobi_damping_factor - 0.4) < 1e-7
    assert c.jacobi_niterations == 5 and c.vcycle_niterations == 6
    assert abs(c.ran_min - 0.01) < 1e-9
    assert c.mg_mode == _lib.MG_REFERENCE and c.mas == _lib.MAS_CIC
    assert c.mg_start == _lib.START_ZERO and abs(c.start_rate - 0.5) < 1e-9


def test_struct_layout_matches_header(lib):
    from baorec import _lib
    # 31 four-byte words; api.cu static_asserts the same size on the C side
    assert ctypes.sizeof(_lib.Config) == 4 * 31
    assert ctypes.sizeof(_lib.SolveStats) == 32
    assert ctypes.sizeof(_lib.GuessTrainConfig) == 4 * 20


def test_field_offsets_match_header(tmp_path):
    """Every field of every struct: offsetof from a C program compiled against
    the header equals the ctypes mirror's offset (and the struct sizes)."""
    import shutil
    import subprocess
    from baorec import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "abi_layout"
    subprocess.run([cc, "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_layout.c"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    mirror = {"baorec_config": _lib.Config, "baorec_solve_stats": _lib.SolveStats,
              "baorec_batch_item": _lib.BatchItem, "baorec_guess_train_config": _lib.GuessTrainConfig,
              "baorec_power_config": _lib.PowerConfig}
    seen = {k: set() for k in mirror}
    for line in out.splitlines():
        st, field, val = line.split()
        cls = mirror[st]
        if field == "sizeof":
            assert ctypes.sizeof(cls) == int(val), st
        else:
            assert getattr(cls, field).offset == int(val), (st, field)
            seen[st].add(field)
    for st, cls in mirror.items():
        assert seen[st] == {name for name, _ in cls._fields_}, st
