"""GPU: the reciprocal and the division of bounded rows (rcp_bounded and
div_bounded in icbc_gb300/csrc/bc1_device.cuh) against the IEEE division.
rcp_bounded equals 1.0f / d for every float d with 2^-100 <= |d| <= 2^100
and for +-0, the range its callers can reach (all 3.4e9 values);
div_bounded equals a / b for every float b in [2^-9, 64] with 16 dividends
each -- 0, seven spread over the floats of [2^-24, 64], eight uniform in
[0, 64) -- its domain (2e9 pairs).  The check program is compiled here with
the encoder's flags."""
import os
import struct
import subprocess
import tempfile

import pytest

from icbc_gb300 import _build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _bits(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def test_bounded_reciprocal_and_division_are_ieee():
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "rcp_check")
        cmd = [_build.nvcc()] + _build.ARCH + _build.NVCC_FLAGS + ["-I", _build.CSRC,
                                                                    os.path.join(HERE, "rcp_check.cu"), "-o", exe]
        subprocess.run(cmd, check=True)
        for mode, lo, hi in (("rcp", _bits(2.0 ** -100), _bits(2.0 ** 100)), ("rcp", 0, 0),
                             ("div", _bits(2.0 ** -9), _bits(64.0))):
            out = subprocess.run([exe, mode, hex(lo), hex(hi)], capture_output=True, text=True,
                                 check=True).stdout.split()
            assert out[0] == "0", "%s: mismatch at bits %s (%d in all)" % (mode, out[1], int(out[0]))
