"""CPU checks of the C-ABI library: it builds for sm_103a, loads without a
GPU, and exports every entry point include/espic.h declares."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, _espic_module


def declared_symbols():
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
            if f.endswith(".h")]
    names = set()
    for h in hdrs:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\bint\s+(espic_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    mod = _espic_module()
    return mod.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "espic_world_create" in names and "espic_step" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_world_create_fails_loudly_without_gpu(libpath):
    mod = _espic_module()
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(mod.EspicError) as e:
        mod.World(5, 5, 5, [0, 0, 0], [1, 1, 1])
    assert "no CUDA device" in str(e.value) or e.value.code == -2
