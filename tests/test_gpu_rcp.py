"""GPU: the reciprocal of the bounded cluster fit (rcp_bounded in
icbc_gb300/csrc/bc1_device.cuh) equals the IEEE division 1.0f / d for every
float d with 2^-100 <= |d| <= 2^100 and for +-0, the range its callers can
reach.  The check program is compiled here with the encoder's flags and runs
over all 3.4e9 values in one launch."""
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


def test_rcp_bounded_is_the_ieee_reciprocal():
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "rcp_check")
        cmd = [_build.nvcc()] + _build.ARCH + _build.NVCC_FLAGS + ["-I", _build.CSRC,
                                                                    os.path.join(HERE, "rcp_check.cu"), "-o", exe]
        subprocess.run(cmd, check=True)
        for lo, hi in ((_bits(2.0 ** -100), _bits(2.0 ** 100)), (0, 0)):
            out = subprocess.run([exe, hex(lo), hex(hi)], capture_output=True, text=True, check=True).stdout.split()
            assert out[0] == "0", "mismatch at bits %s (%d in all)" % (out[1], int(out[0]))
