"""CPU: the fused forms of the encoder's arithmetic give the bits of the
unfused IEEE sequences they replace (tests/fused_forms_check.c): the 565
snap's multiply-add for every float in [0, 1], and the bounded rows'
division sequence over its domain (every 16th divisor here; every divisor
on the GPU with the device reciprocal, tests/test_gpu_rcp.py)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(*args):
    cc = shutil.which(os.environ.get("CC", "gcc"))
    if not cc:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "fused_forms_check")
        subprocess.run([cc, "-O2", "-std=c99", "-ffp-contract=off", "-fno-fast-math",
                        os.path.join(HERE, "fused_forms_check.c"), "-o", exe, "-lm"], check=True)
        return subprocess.run([exe, *args], capture_output=True, text=True, check=True).stdout.strip()


def test_snap_fma_equals_unfused_floor():
    assert _run("snap") == "0"


def test_bounded_division_sequence_equals_ieee():
    assert _run("div", "16") == "0"
