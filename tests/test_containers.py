"""DDS / KTX writers and the golden-file compare (icbc_test.cpp:155-279):
host-side tests on CPU, device-resident blocks on the GPU."""
import os
import struct

import numpy as np
import pytest

import icbc_gb300 as ig


def _blocks(w, h, seed=0):
    n = ((w + 3) // 4) * ((h + 3) // 4)
    return (np.arange(n * 8, dtype=np.uint64) * 2654435761 + seed).astype(np.uint8).reshape(n, 8)


def test_dds_layout_and_compare(tmp_path):
    w, h = 70, 45
    b = _blocks(w, h)
    path = str(tmp_path / "img_bc1.dds")
    ig.write_dds(path, w, h, b)
    data = open(path, "rb").read()
    assert len(data) == 128 + b.size
    magic, size, flags, height, width, linear, depth, mips = struct.unpack("<4s7I", data[:32])
    assert (magic, size, height, width, linear, mips) == (b"DDS ", 124, h, w, b.size, 1)
    assert flags == 0x1 | 0x1000 | 0x4 | 0x2 | 0x80000
    pf_size, pf_flags, pf_fourcc = struct.unpack("<II4s", data[76:88])
    assert (pf_size, pf_flags, pf_fourcc) == (32, 4, b"DXT1")
    assert struct.unpack("<I", data[108:112])[0] == 0x1000
    assert data[128:] == b.tobytes()
    assert ig.compare_dds(path, w, h, b)
    b2 = b.copy()
    b2[7, 3] ^= 1
    assert not ig.compare_dds(path, w, h, b2)
    with pytest.raises(ig.IcbcGpuError):
        ig.compare_dds(str(tmp_path / "missing.dds"), w, h, b)


def test_ktx_layout(tmp_path):
    w, h = 64, 32
    b = _blocks(w, h, 3)
    path = str(tmp_path / "img_bc1.ktx")
    ig.write_ktx(path, w, h, b)
    data = open(path, "rb").read()
    assert data[:12] == bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
    fields = struct.unpack("<13I", data[12:64])
    assert fields[0] == 0x04030201 and fields[4] == 0x83F0 and fields[5] == 0x1908
    assert fields[6:9] == (w, h, 0) and fields[10:12] == (1, 1)
    assert struct.unpack("<I", data[64:68])[0] == b.size
    assert data[68:] == b.tobytes()


@pytest.mark.gpu
def test_dds_from_device_blocks(gpu_lib, tmp_path):
    import torch
    from icbc_gb300 import synth
    img = synth.gradient_noise_rects(96, 64, 2)
    out = gpu_lib.compress_image(torch.from_numpy(img).cuda(), 8, 0)
    path = str(tmp_path / "dev.dds")
    gpu_lib.write_dds(path, 96, 64, out)
    assert gpu_lib.compare_dds(path, 96, 64, out.cpu().numpy())
    assert gpu_lib.compare_dds(path, 96, 64, out)


def test_dds_mip_chain_layout(tmp_path):
    w, h = 37, 21
    levels = ig.mip_levels(w, h)
    assert levels == 6  # 37x21, 18x10, 9x5, 4x2, 2x1, 1x1
    ws, hs, off = ig.mip_layout(w, h)
    assert (ws, hs) == ([37, 18, 9, 4, 2, 1], [21, 10, 5, 2, 1, 1])
    assert off == [0, 60, 75, 81, 82, 83, 84]
    b = _blocks(100, 100)[: off[-1]]
    path = str(tmp_path / "mips.dds")
    ig.write_dds_mips(path, w, h, levels, b)
    data = open(path, "rb").read()
    assert len(data) == 128 + 8 * off[-1]
    magic, size, flags, height, width, linear, depth, mips = struct.unpack("<4s7I", data[:32])
    assert (magic, height, width, linear, mips) == (b"DDS ", h, w, 8 * off[1], levels)
    assert flags & 0x20000  # DDSD_MIPMAPCOUNT
    assert struct.unpack("<I", data[108:112])[0] == 0x1000 | 0x400000 | 0x8
    assert data[128:] == b.tobytes()
