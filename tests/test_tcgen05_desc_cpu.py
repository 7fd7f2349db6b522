"""Host-side encoders of the tcgen05 descriptors (lywell_gb300/csrc/mlf_tcgen05.h)
against encodings worked out by hand from the PTX ISA's bit layouts.  No GPU:
the header is compiled with the host C++ compiler.

Shared-memory matrix descriptor (64 bits): start address >> 4 in [0,14),
leading byte offset >> 4 in [16,30), stride byte offset >> 4 in [32,46),
version 1 in [46,48), base offset [49,52), swizzle mode in [61,64)
(2 = 128-byte).  Instruction descriptor (32 bits): D format [4,6) (1 = F32),
A / B format [7,10) / [10,13) (1 = BF16, 2 = TF32), majors [15], [16]
(0 = K), N >> 3 in [17,23), M >> 4 in [24,29).
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = r"""
#include <cstdio>
#include "mlf_tcgen05.h"
using namespace mlf::tc;
int main() {
    std::printf("%016llx\n", (unsigned long long)kmajor_sw128_desc(0x1400));
    std::printf("%016llx\n", (unsigned long long)kmajor_sw128_desc(0x1400 + 96));
    std::printf("%016llx\n", (unsigned long long)smem_desc(0x2000, 128, 256, SWIZZLE_NONE));
    std::printf("%08x\n", instr_desc_f32acc(FMT_TF32, 128, 160));
    std::printf("%08x\n", instr_desc_f32acc(FMT_BF16, 128, 256));
    std::printf("%08x\n", instr_desc_f32acc(FMT_TF32, 64, 8));
    std::printf("%d %d %d %d %d\n", valid_shape(128, 160), valid_shape(128, 8), valid_shape(64, 8),
                valid_shape(128, 272), valid_shape(256, 64));
    std::printf("%u %u %u %u\n", sw128_offset(0, 0), sw128_offset(1, 0), sw128_offset(9, 3), sw128_offset(7, 7));
    std::printf("%08x\n", instr_desc_f32acc(FMT_BF16, 128, 128));
    return 0;
}
"""


@pytest.fixture(scope="module")
def encodings(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("tcdesc")
    src = d / "t.cpp"
    src.write_text(SRC)
    exe = d / "t"
    subprocess.run([cxx, "-std=c++17", "-I", os.path.join(ROOT, "lywell_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")


def test_smem_descriptor_kmajor_sw128(encodings):
    # 0x1400 >> 4 = 0x140; LBO 16 B -> 1 << 16; SBO 1024 B -> 64 << 32;
    # version 1 << 46; 128-byte swizzle 2 << 61
    assert int(encodings[0], 16) == 0x140 | (1 << 16) | (64 << 32) | (1 << 46) | (2 << 61)
    assert int(encodings[0], 16) == 0x4000404000010140
    # a K step of 24 TF32 (96 bytes) inside the swizzle atom moves only the start address
    assert int(encodings[1], 16) == 0x4000404000010146


def test_smem_descriptor_no_swizzle(encodings):
    assert int(encodings[2], 16) == 0x200 | (8 << 16) | (16 << 32) | (1 << 46)


def test_instruction_descriptor(encodings):
    # F32 accumulator (1 << 4), TF32 A and B (2 << 7, 2 << 10), N = 160 (20 << 17), M = 128 (8 << 24)
    assert int(encodings[3], 16) == 0x08280910
    # BF16 A and B (1 << 7, 1 << 10), N = 256 (32 << 17), M = 128
    assert int(encodings[4], 16) == 0x08400490
    # M = 64 (4 << 24), N = 8 (1 << 17)
    assert int(encodings[5], 16) == (1 << 4) | (2 << 7) | (2 << 10) | (1 << 17) | (4 << 24)


def test_valid_shapes(encodings):
    assert encodings[6].split() == ["1", "0", "1", "0", "0"]


def test_sw128_chunk_offsets(encodings):
    # row 0 chunk 0 in place; row 1 chunk 0 -> chunk 1 (128 + 16); row 9 (atom 1, row 1 of
    # it) chunk 3 -> chunk 2 (9 * 128 + 32); row 7 chunk 7 -> chunk 0 (7 * 128)
    assert encodings[7].split() == ["0", "144", "1184", "896"]


def test_instruction_descriptor_bf16_square(encodings):
    # BF16 A and B (1 << 7, 1 << 10), F32 D, N = 128 (16 << 17), M = 128 (8 << 24)
    assert int(encodings[8], 16) == (1 << 4) | (1 << 7) | (1 << 10) | (16 << 17) | (8 << 24)
