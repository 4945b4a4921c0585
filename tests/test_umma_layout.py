"""CPU checks of the tcgen05 one-pass kernel's shared-memory, descriptor and
tensor-memory arithmetic (csrc/kernels_umma.cu), mirrored here and asserted
against the source constants, so that every address the kernel forms is
checked before it runs on a GPU:

* shared-memory regions lie inside the dynamic allocation, do not overlap and
  are aligned as the 64-byte swizzle (512-byte atoms) and the barriers need;
* the producers' swizzled 16-byte digit stores land exactly where the
  tensor core reads element (row, k) of a K-major, 64-byte-swizzled operand
  through the kernel's descriptors (start address, SBO = 512, k16 offset);
* every MMA's shared-memory reads stay inside its plane / stage region and
  its TMEM columns inside the allocation; N is a legal kind::f16 width for
  M = 128; the instruction and matrix descriptor fields hold what they encode;
* the epilogue's TMEM addresses stay in the warp's lane quadrant.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = open(os.path.join(ROOT, "zmpo_dmrg_gb300", "csrc", "kernels_umma.cu")).read()
COMMON = open(os.path.join(ROOT, "zmpo_dmrg_gb300", "csrc", "device_common.cuh")).read()

TM, KMAX, KB_SLOTS, ROW_BYTES, NSTAGE, NTHREADS = 128, 256, 32, 64, 2, 416
EPI_WARPS, PROD_WARP0, PROD_WARPS, MMA_WARP = 4, 4, 8, 12
SLOT_BYTES = 56
SMEM_MAX = 232448


def test_constants_match_source():
    for name, val in [("TM", TM), ("KMAX", KMAX), ("KB_SLOTS", KB_SLOTS), ("ROW_BYTES", ROW_BYTES),
                      ("NSTAGE", NSTAGE), ("NTHREADS", NTHREADS)]:
        assert re.search(r"constexpr int %s = %d;" % (name, val), SRC), name
    assert "EPI_WARPS = 4, PROD_WARP0 = 4, PROD_WARPS = 8, MMA_WARP = 12" in SRC
    assert (EPI_WARPS + PROD_WARPS + 1) * 32 == NTHREADS
    # Slot: two pointers, two int64, one double, four ints
    body = re.search(r"struct Slot \{(.*?)\};", COMMON, re.S).group(1)
    assert re.findall(r"const double \*(\w+);", body) == ["a", "b"]
    assert "int64_t sam, sbn;" in body and "double alpha;" in body
    assert len(re.findall(r"\bint (\w+);", body)) == 4


def layout(TN):
    L = {}
    L["B_KB"] = 4 * TN * ROW_BYTES
    L["OFF_B"] = 0
    L["OFF_A"] = L["OFF_B"] + (KMAX // KB_SLOTS) * L["B_KB"]
    L["A_PLANE"] = TM * ROW_BYTES
    L["A_STAGE"] = 4 * L["A_PLANE"]
    L["OFF_SLOTS"] = L["OFF_A"] + NSTAGE * L["A_STAGE"]
    L["OFF_REC"] = L["OFF_SLOTS"] + KMAX * SLOT_BYTES
    L["REC_EA"] = 0
    L["REC_EB"] = TM * 4
    L["REC_CB"] = L["REC_EB"] + TN * 4
    L["REC_RS"] = L["REC_CB"] + TN * 8
    L["REC_INFO"] = L["REC_RS"] + TN * 8
    L["REC_BYTES"] = L["REC_INFO"] + 16
    L["OFF_ITEM"] = L["OFF_REC"] + 2 * L["REC_BYTES"]
    L["ITEM_BYTES"] = TN * 4 + TN * 16
    L["OFF_BAR"] = (L["OFF_ITEM"] + L["ITEM_BYTES"] + 7) // 8 * 8
    L["OFF_MISC"] = L["OFF_BAR"] + 15 * 8
    L["BYTES"] = L["OFF_MISC"] + 16
    L["SMEM"] = L["BYTES"] + 1024
    L["TMEM_COLS"] = 8 * TN
    return L


def test_layout_formulas_match_source():
    for expr in ["B_KB = 4 * TN * ROW_BYTES", "OFF_A = OFF_B + NKB_MAX * B_KB",
                 "OFF_SLOTS = OFF_A + NSTAGE * A_STAGE", "OFF_REC = OFF_SLOTS + KMAX * (int)sizeof(Slot)",
                 "REC_EB = REC_EA + TM * 4", "REC_CB = REC_EB + TN * 4", "REC_RS = REC_CB + TN * 8",
                 "REC_INFO = REC_RS + TN * 8", "REC_BYTES = REC_INFO + 16", "OFF_ITEM = OFF_REC + 2 * REC_BYTES",
                 "ITEM_BYTES = TN * 4 + TN * 16", "OFF_BAR = (OFF_ITEM + ITEM_BYTES + 7) / 8 * 8",
                 "NBAR = 15", "OFF_MISC = OFF_BAR + NBAR * 8", "BYTES = OFF_MISC + 16", "SMEM = BYTES + 1024",
                 "TMEM_COLS = 8 * TN", "A_PLANE = TM * ROW_BYTES", "A_STAGE = 4 * A_PLANE"]:
        assert expr in SRC, expr


@pytest.mark.parametrize("TN", [16, 32, 64])
def test_shared_memory_regions(TN):
    L = layout(TN)
    assert L["SMEM"] <= SMEM_MAX
    regions = [("B", L["OFF_B"], L["OFF_A"]), ("A", L["OFF_A"], L["OFF_SLOTS"]),
               ("slots", L["OFF_SLOTS"], L["OFF_REC"]), ("rec", L["OFF_REC"], L["OFF_REC"] + 2 * L["REC_BYTES"]),
               ("item", L["OFF_ITEM"], L["OFF_ITEM"] + L["ITEM_BYTES"]),
               ("bar", L["OFF_BAR"], L["OFF_BAR"] + 15 * 8), ("misc", L["OFF_MISC"], L["OFF_MISC"] + 16)]
    for (_, a0, a1), (_, b0, b1) in zip(regions, regions[1:]):
        assert a0 <= a1 <= b0 <= b1
    assert regions[-1][2] <= L["BYTES"]
    # base aligned to 1024 at run time: 1023 bytes of slack at most
    assert L["BYTES"] + 1023 <= L["SMEM"]
    assert L["OFF_A"] % 1024 == 0 and L["A_STAGE"] % 1024 == 0 and L["B_KB"] % 512 == 0
    assert L["A_PLANE"] % 512 == 0 and (TN * ROW_BYTES) % 512 == 0
    assert L["OFF_BAR"] % 8 == 0 and L["OFF_SLOTS"] % 16 == 0 and L["OFF_REC"] % 16 == 0
    assert (L["OFF_REC"] + L["REC_CB"]) % 8 == 0 and (L["OFF_ITEM"] + TN * 4) % 8 == 0
    # one CTA per SM: two would need more shared memory than an SM has, or
    # fit in TMEM together (no blocking allocation)
    assert 2 * L["SMEM"] > 228 * 1024 or 2 * L["TMEM_COLS"] <= 512
    assert L["TMEM_COLS"] in (32, 64, 128, 256, 512)


def store_offset(row, chunk):
    """cut8_store: byte offset of 16-byte chunk `chunk` of `row` in a plane."""
    return row * ROW_BYTES + ((chunk ^ ((row >> 1) & 3)) << 4)


def tensor_core_read(start, row, k):
    """Byte address the tensor core reads element (row, k), k < 16, of a
    K-major operand with 64-byte swizzle from a descriptor at `start`
    (SBO = 512): rows at 64-byte pitch in 8-row groups, 16-byte chunk bits
    [4, 6) XOR address bits [7, 9)."""
    a = start + (row // 8) * 512 + (row % 8) * 64 + (k // 8) * 16 + (k % 8) * 2
    return a ^ (((a >> 7) & 3) << 4)


@pytest.mark.parametrize("TN", [16, 32, 64])
def test_swizzled_stores_match_descriptor_reads(TN):
    L = layout(TN)
    base = 1024 * 7   # any 1024-aligned dynamic-smem base
    # A: stage s, plane p, row r, slot j
    for s in range(NSTAGE):
        for p in range(4):
            plane = base + L["OFF_A"] + s * L["A_STAGE"] + p * L["A_PLANE"]
            for r in range(TM):
                for j in range(KB_SLOTS):
                    w = plane + store_offset(r, j // 8) + (j % 8) * 2
                    k16, k = divmod(j, 16)
                    assert tensor_core_read(plane + k16 * 32, r, k) == w
                    assert plane <= w < plane + L["A_PLANE"]
    # B': k block kb, plane p, column c -> operand row p*TN + c
    for kb in range(KMAX // KB_SLOTS):
        blk = base + L["OFF_B"] + kb * L["B_KB"]
        for p in range(4):
            for c in range(TN):
                for j in range(KB_SLOTS):
                    w = blk + p * TN * ROW_BYTES + store_offset(c, j // 8) + (j % 8) * 2
                    k16, k = divmod(j, 16)
                    assert tensor_core_read(blk + k16 * 32, p * TN + c, k) == w
                    assert blk <= w < blk + L["B_KB"]


@pytest.mark.parametrize("TN", [16, 32, 64])
def test_mma_operand_and_tmem_ranges(TN):
    L = layout(TN)
    for a in range(4):
        n = (4 - a) * TN
        assert n % 16 == 0 and 16 <= n <= 256            # kind::f16, M = 128
        # B operand rows [0, n) of a k block: inside the block
        assert n * ROW_BYTES <= L["B_KB"]
        # A operand: plane a of a stage, 128 rows
        assert (a + 1) * L["A_PLANE"] <= L["A_STAGE"]
        for b in range(2):
            col0 = b * 4 * TN + a * TN
            assert col0 + n <= L["TMEM_COLS"]
    # epilogue reads: buffer b, level l, 16 columns at c0
    for b in range(2):
        for l in range(4):
            for c0 in range(0, TN, 16):
                assert b * 4 * TN + l * TN + c0 + 16 <= L["TMEM_COLS"]
    # descriptor start address field: 14 bits of (addr >> 4)
    assert (L["SMEM"] + 1024) >> 4 < (1 << 14)


def test_descriptor_encodings():
    def idesc(n, m=128):
        return (1 << 4) | (1 << 7) | (1 << 10) | ((n >> 3) << 17) | ((m >> 4) << 24)
    src = re.search(r"uint32_t idesc\(int n\) \{(.*?)\}", SRC, re.S).group(1)
    assert "(1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TM >> 4) << 24)" in src
    for n in (16, 32, 48, 64, 96, 128, 192, 256):
        d = idesc(n)
        assert (d >> 4) & 3 == 1          # D: F32
        assert (d >> 7) & 7 == 1          # A: BF16
        assert (d >> 10) & 7 == 1         # B: BF16
        assert (d >> 15) & 3 == 0         # both K-major
        assert (d >> 17) & 63 == n >> 3
        assert (d >> 24) & 31 == 8        # M = 128
        assert d & 0b1111 == 0 and (d >> 13) & 3 == 0 and (d >> 23) & 1 == 0 and d >> 29 == 0
    sd = re.search(r"uint64_t sdesc\(uint32_t addr\) \{(.*?)\}", SRC, re.S).group(1)
    assert "((uint64_t)(512u >> 4) << 32)" in sd and "((uint64_t)1u << 46)" in sd and "((uint64_t)4u << 61)" in sd
