"""CPU: the multiply-add-shift palette constants the encoder uses for the
D3D10, AMD and Intel decoders equal the reference's integer formulas
(icbc.h:2752-2874) for every pair of 8-bit endpoint channels.  The constants
are read from the library source so the check cannot drift from the code."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "icbc_gb300", "csrc",
                   "icbc_gpu_api.cu")


def constants():
    text = open(SRC).read()
    block = re.search(r"kLin\[4\]\[8\] = \{(.*?)\};", text, re.S).group(1)
    rows = re.findall(r"\{([^{}]*)\}", block)
    return [[int(x) for x in r.split(",")] for r in rows]


def test_linear_palette_forms_exact():
    lin = constants()
    a, b = np.meshgrid(np.arange(256, dtype=np.int64), np.arange(256, dtype=np.int64), indexing="ij")
    ref4 = {0: (2 * a + b) // 3, 2: (43 * a + 21 * b + 32) >> 6, 3: (171 * a + 85 * b + 128) >> 8}
    ref3 = {0: (a + b) // 2, 2: (a + b + 1) // 2, 3: (128 * a + 128 * b + 128) >> 8}
    for d in (0, 2, 3):
        ma, mb, rd, sh, ca, cb, r3, s3 = lin[d]
        assert np.array_equal((ma * a + mb * b + rd) >> sh, ref4[d]), d
        assert np.array_equal((ca * a + cb * b + r3) >> s3, ref3[d]), d
        assert (ma * 255 + mb * 255 + rd) < 2 ** 31
