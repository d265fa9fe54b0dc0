"""The C-ABI library loads and exports every entry point of include/mcacg.h."""
import ctypes
import re

import pytest

from conftest import ROOT


def header_functions():
    text = (ROOT / "include" / "mcacg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mcacg_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(built_library):
    lib = ctypes.CDLL(str(built_library))
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from mcac_gb300 import _lib
    assert set(header_functions()) == set(_lib.SIGNATURES)


def test_abi_version_and_errors():
    from mcac_gb300 import _lib
    lib = _lib.lib()
    assert lib.mcacg_abi_version() == 2
    # a null argument is rejected with a status, not a crash
    assert lib.mcacg_params_default(None) == 103
    assert b"null" in lib.mcacg_last_error()


def test_merge_grid_threshold_setting():
    """The all-pairs / cell-grid switch of the merge is a process-wide
    setting: positive sizes only, the previous value returned."""
    from mcac_gb300 import set_merge_grid_min
    from mcac_gb300._lib import MCACError
    with pytest.raises(MCACError):
        set_merge_grid_min(0)
    prev = set_merge_grid_min(64)
    try:
        assert prev == 2048
        assert set_merge_grid_min(128) == 64
    finally:
        set_merge_grid_min(prev)
