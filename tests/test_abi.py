"""The C ABI library loads and exports every entry point include/stater.h declares."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "stater.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(stater_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from stater_gb300 import build as b
    b.build()
    import stater_gb300
    return stater_gb300.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("stater_setup", "stater_denoise_vars", "stater_denoise_film", "stater_calc_target_spp",
              "stater_synchronize", "stater_print_macro_configuration", "stater_accumulate"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_host_only_entry_points(lib):
    import ctypes
    import numpy as np
    assert lib.stater_abi_version() == 2
    n = lib.stater_tcrit_lut_intervals()
    t = np.zeros(n + 1)
    assert lib.stater_tcrit2_table(ctypes.c_double(0.01), t.ctypes.data_as(ctypes.c_void_p)) == 0
    import oracle
    assert np.allclose(t, oracle.tcrit2_table(0.01, n), rtol=1e-13)
    assert lib.stater_tcrit2_table(ctypes.c_double(1.5), t.ctypes.data_as(ctypes.c_void_p)) == 1
    assert b"alpha" in lib.stater_last_error()
