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


def test_entry_points_refuse_a_null_world(libpath):
    """The ch4 entry points (DSMC, moments, MCC, neutral push) return an
    argument error with a message for a null world handle, on any host."""
    L = ctypes.CDLL(libpath)
    L.espic_last_error.argtypes = [ctypes.c_char_p, ctypes.c_int]
    null = ctypes.c_void_p(None)
    calls = {
        "espic_dsmc_enable": (null, 0, None, ctypes.c_double(1e-14)),
        "espic_dsmc_apply": (null, 0, ctypes.c_double(1e-7), None, ctypes.c_int64(0), None),
        "espic_dsmc_status": (null, 0, None, None, None),
        "espic_sample_moments": (null, 0),
        "espic_gas_properties": (null, 0),
        "espic_clear_samples": (null, 0),
        "espic_compute_mpc": (null, 0),
        "espic_mcc_cex": (null, 0, 1, ctypes.c_double(1e-7), None, ctypes.c_int64(0), None, None),
        "espic_advance_ch4": (null, 0, None, None, ctypes.c_int64(0), None, None),
    }
    for name, args in calls.items():
        rc = getattr(L, name)(*args)
        assert rc < 0, name
        buf = ctypes.create_string_buffer(256)
        L.espic_last_error(buf, 256)
        assert b"null world" in buf.value, (name, buf.value)


def test_noalloc_refuses_oversized_grids_before_any_work(libpath):
    """espic_deposit_noalloc bounds each axis before multiplying: grids whose
    node count would wrap a 64-bit product (2^22 x 2^21 x 2^21 wraps to 0,
    (2^21)^3 to a negative value) are refused like any grid beyond the
    static scratch, without touching the GPU (so this runs on any host)."""
    L = ctypes.CDLL(libpath)
    L.espic_last_error.argtypes = [ctypes.c_char_p, ctypes.c_int]
    f = L.espic_deposit_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    x0 = (ctypes.c_double * 3)(0, 0, 0)
    xm = (ctypes.c_double * 3)(1, 1, 1)
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the call refuses first
    for dims in [(1 << 22, 1 << 21, 1 << 21), (1 << 21, 1 << 21, 1 << 21), (1 << 20, 1 << 20, 4),
                 (2**31 - 1, 3, 3), (102, 103, 101)]:
        rc = f(None, 0, 0, *dims, x0, xm, 1.0, fake, None, None)
        assert rc == -1, dims
        buf = ctypes.create_string_buffer(256)
        L.espic_last_error(buf, 256)
        assert b"scratch" in buf.value, (dims, buf.value)
