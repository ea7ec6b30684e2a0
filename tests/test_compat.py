"""The C++ drop-in (include/icbc_compat.hpp): code written against icbc's own
header links against libicbc_gpu.so unchanged and gets the reference's
results."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import icbc_gb300 as ig
from icbc_gb300 import synth
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_HEADER_DIR = O.reference_dir()


def _cxx():
    return shutil.which(os.environ.get("CXX", "g++"))


@pytest.mark.skipif(not REF_HEADER_DIR or not _cxx(),
                    reason="reference header or C++ compiler not available")
def test_reference_header_symbols_resolve():
    """Every icbc:: symbol a caller compiled against the reference's icbc.h
    needs is defined by the library."""
    lib = ig._build.build()
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "caller.cpp")
        with open(src, "w") as f:
            f.write('#include "icbc.h"\n'
                    'float use(const float *c, const float *w, const float *cw, void *o, unsigned char *t) {\n'
                    '  icbc::init(icbc::Decoder_NVIDIA);\n'
                    '  icbc::decode_bc1(o, t);\n'
                    '  icbc::decode_bc3(o, t, icbc::Decoder_Intel);\n'
                    '  return icbc::compress_bc1(icbc::Quality_Max, c, w, cw, true, true, o) +\n'
                    '         icbc::evaluate_bc1_error(t, o, icbc::Decoder_AMD) +\n'
                    '         icbc::evaluate_bc3_error(t, o, true) +\n'
                    '         icbc::compress_bc3(icbc::Quality_Level4, c, w, cw, false, o);\n}\n')
        obj = os.path.join(tmp, "caller.o")
        subprocess.run([_cxx(), "-c", "-I", REF_HEADER_DIR, src, "-o", obj], check=True)
        need = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout.split()
        need = {s for s in need if "icbc" in s}
        have = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True,
                              check=True).stdout.split()
        assert need and need <= set(have), need - set(have)


@pytest.mark.gpu
def test_cpp_dropin_matches_oracle(gpu_lib):
    if not _cxx():
        pytest.skip("no C++ compiler")
    lib = ig._build.build()
    cols, w = synth.mixed_blocks(96, seed=41)
    rgba = np.concatenate([(cols[:, :, :3] * 255.0 + 0.5).astype(np.uint8),
                           np.full((96, 16, 1), 255, np.uint8)], axis=2)
    levels = [0, 4, 8, 9]
    decoder, cw = 2, np.array([0.299, 0.587, 0.114], np.float32)
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "driver")
        subprocess.run([_cxx(), "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests",
                        "compat_driver.cpp"), lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
        inp, outp = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        with open(inp, "wb") as f:
            f.write(np.array([96, decoder, len(levels)] + levels, np.int32).tobytes())
            f.write(cw.tobytes())
            for i in range(96):
                f.write(cols[i].tobytes() + w[i].tobytes() + rgba[i].tobytes())
        subprocess.run([exe, inp, outp], check=True)
        data = np.fromfile(outp, np.uint8)
    pos = 0
    blocks = None
    for lv in levels:
        rec = data[pos:pos + 96 * 12].reshape(96, 12)
        pos += 96 * 12
        blocks = rec[:, :8]
        errs = rec[:, 8:].copy().view(np.float32).reshape(96)
        ob, oe = O.compress_blocks(cols, w, lv, decoder, cw, True, True)
        assert np.array_equal(blocks, ob), lv
        assert np.array_equal(errs.view(np.uint32), oe.view(np.uint32)), lv
    rec = data[pos:pos + 96 * 68].reshape(96, 68)
    pos += 96 * 68
    assert np.array_equal(rec[:, :64], O.decode_bc1(blocks, decoder))
    ev = rec[:, 64:].copy().view(np.float32).reshape(96)
    assert np.array_equal(ev.view(np.uint32), O.evaluate_bc1_error(rgba.reshape(96, 64), blocks, decoder).view(np.uint32))
    # BC3 as the reference has it: decode / evaluate, and compress_bc3 = 0 with the block untouched
    i = np.arange(96, dtype=np.uint8)
    bc3 = np.concatenate([i[:, None], (255 - i)[:, None], np.repeat(i[:, None], 6, 1), blocks], axis=1)
    rec = data[pos:pos + 96 * 73].reshape(96, 73)
    assert pos + 96 * 73 == data.size
    assert np.array_equal(rec[:, :64], O.decode_bc3(bc3, decoder))
    e3 = rec[:, 64:68].copy().view(np.float32).reshape(96)
    assert np.array_equal(e3.view(np.uint32), O.evaluate_bc3_error(rgba.reshape(96, 64), bc3, True, decoder).view(np.uint32))
    assert np.all(rec[:, 68:72].copy().view(np.float32) == 0.0) and np.all(rec[:, 72] == 1)
