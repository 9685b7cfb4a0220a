"""C-ABI library checks that need no GPU: it loads, exports every symbol
include/xcorr.h declares, and its pure host functions behave."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

import xcorr


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "xcorr.h")).read()
    return sorted(set(re.findall(r"\b(xc_[a-z0-9_]+)\s*\(", text)))


def test_library_built_and_loads():
    assert os.path.exists(xcorr.LIB_PATH), "run __graft_entry__.build() first"
    assert xcorr.lib().xc_version().decode().startswith("xcorr-gb300")


def test_every_declared_symbol_is_exported():
    L = ctypes.CDLL(xcorr.LIB_PATH)
    decl = declared_symbols()
    assert len(decl) >= 30
    missing = [s for s in decl if not hasattr(L, s)]
    assert not missing, missing
    assert sorted(xcorr.EXPORTED) == decl


def test_output_count_modes():
    assert xcorr.output_count("one_to_one", 1, 1) == 1
    assert xcorr.output_count("one_to_many", 1, 64) == 64
    assert xcorr.output_count("n_to_mn", 8, 32) == 32
    assert xcorr.output_count("n_to_m", 8, 32) == 256


@pytest.mark.parametrize("mode,n,m", [("one_to_one", 2, 1), ("one_to_many", 2, 3), ("n_to_mn", 3, 4),
                                      ("n_to_m", 0, 4), ("one_to_one", 0, 0)])
def test_output_count_rejects_invalid(mode, n, m):
    with pytest.raises(xcorr.XcError) as e:
        xcorr.output_count(mode, n, m)
    assert e.value.status == 1
    assert "invalid" in str(e.value)


def test_output_size_and_workspace():
    out = xcorr.Size2()
    xcorr.check(xcorr.lib().xc_output_size(xcorr.size2(23, 37), xcorr.size2(9, 14), ctypes.byref(out)))
    assert (out.y, out.x) == (31, 50)
    assert xcorr.workspace_size("one_to_many", "f32", "direct", (256, 256), 1, (256, 256), 64) == 0
    fft = xcorr.workspace_size("one_to_many", "f32", "fft", (256, 256), 1, (256, 256), 64)
    # 65 input spectra + 64 products of 512 x 257 complex floats
    assert fft >= (65 + 64) * 512 * 257 * 8
    with pytest.raises(xcorr.XcError):
        xcorr.lib_call = xcorr.check(xcorr.lib().xc_output_size(xcorr.size2(0, 5), xcorr.size2(3, 3),
                                                                ctypes.byref(out)))


def test_status_strings():
    L = xcorr.lib()
    assert L.xc_status_string(0) == b"ok"
    assert L.xc_status_string(6) == b"device wait timed out"
