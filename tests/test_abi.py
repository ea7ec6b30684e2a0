"""CPU: the C-ABI library builds, loads without a GPU, exports every symbol
the public headers declare, and its host-built init tables equal the
oracle's (no compute call is made)."""
import ctypes
import os
import re

import numpy as np
import pytest

import icbc_gb300 as ig
from icbc_gb300 import _build
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(icbc_gpu_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    return ig.load()


def test_header_symbols_exported(lib):
    names = declared_functions("icbc_gpu.h")
    assert len(names) >= 15
    dll = ctypes.CDLL(_build.LIB_PATH)
    missing = [n for n in names if not hasattr(dll, n)]
    assert not missing, missing


def test_status_strings(lib):
    for code in range(10):
        assert lib.icbc_gpu_status_string(code)
    assert lib.icbc_gpu_get_decoder() in (-1, 0, 1, 2, 3)


@pytest.mark.parametrize("decoder", range(4))
def test_host_tables_equal_oracle(lib, decoder):
    t = ig.debug_tables(decoder)
    m5, m6, w = O.tables(decoder)
    assert np.array_equal(t["match5"], m5)
    assert np.array_equal(t["match6"], m6)
    assert np.array_equal(t["weights"].view(np.uint32), w.view(np.uint32))
    four, ft, three, tt = O.cluster_tables()
    assert np.array_equal(t["four"], four)
    assert np.array_equal(t["four_total"], ft)
    assert np.array_equal(t["three"], three)
    assert np.array_equal(t["three_total"], tt)


def test_invalid_arguments_rejected_without_launch(lib):
    cw = (ctypes.c_float * 3)(1, 1, 1)
    # bad level, bad size: rejected before any CUDA call
    assert lib.icbc_gpu_compress_bc1_blocks(10, None, None, cw, 1, 1, 0, None, None, 1, None) == 1
    assert lib.icbc_gpu_compress_bc1_blocks(0, None, None, cw, 1, 1, 0, None, None, -1, None) == 1
    assert lib.icbc_gpu_compress_bc1_blocks(0, None, None, cw, 1, 1, 0, None, None, 0, None) == 0
    assert lib.icbc_gpu_init(7) == 1
    assert lib.icbc_gpu_decode_bc1(None, None, -5, 0, None) == 1
    d = ig.ImageDesc()
    assert lib.icbc_gpu_compress_bc1_image(ctypes.byref(d), None) == 1
