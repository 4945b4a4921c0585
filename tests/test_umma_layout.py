"""CPU checks of the tcgen05 one-pass path's shared-memory, plane-record,
descriptor and tensor-memory arithmetic (csrc/kernels_umma.cu, the record
sizes in csrc/engine.h), mirrored here and asserted against the source
constants, so that every address the kernels form is checked before it runs
on a GPU:

* shared-memory regions lie inside the dynamic allocation, do not overlap and
  are aligned as the 64-byte swizzle (512-byte atoms), the bulk copies
  (16 bytes) and the barriers need;
* the prepare kernels' swizzled 16-byte digit stores into a tile record land,
  once the record is bulk-copied into its shared-memory stage, exactly where
  the tensor core reads element (row, k) of a K-major, 64-byte-swizzled
  operand through the kernel's descriptors (start address, SBO = 512, k16
  offset);
* the exponent / column-map parts of the records land in the tile record's
  fields; every bulk copy is 16-byte aligned and sized, and the bytes a
  barrier phase expects stay within the transaction-count range;
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
ENGINE = open(os.path.join(ROOT, "zmpo_dmrg_gb300", "csrc", "engine.h")).read()
PLANNER = open(os.path.join(ROOT, "zmpo_dmrg_gb300", "csrc", "planner.cpp")).read()

TM, KMAX, KB_SLOTS, ROW_BYTES, NTHREADS = 128, 256, 32, 64, 576
EPI_WARPS, PROD_WARP, MMA_WARP = 16, 16, 17
STG_BYTES = EPI_WARPS * 32 * 4 * 8
SMEM_MAX = 232448
TX_MAX = (1 << 20) - 1


NKBBS = (8, 4, 2)   # B k blocks of the one-pass launches (a launch per class)


BAR_A_FULL = 13


def nbb(TN, NKBB):
    """B buffers of the one-pass kernel: two when two fit next to a ring of at
    least two A stages."""
    b_kb = 4 * TN * ROW_BYTES
    rec = TM * 4 + TN * 20 + 16
    free = SMEM_MAX - 1024 - 2 * rec - STG_BYTES - 16 - 8 * (BAR_A_FULL + 2 * 6)
    return 2 if free - 2 * NKBB * b_kb >= 2 * 4 * TM * ROW_BYTES else 1


def nstage(TN, NKBB):
    """A ring of the one-pass kernel: as many 32 KB stages as the rest of the
    227 KB leaves (at most 6) next to the B buffers of NKBB k blocks."""
    b_kb = 4 * TN * ROW_BYTES
    rec = TM * 4 + TN * 20 + 16
    free = SMEM_MAX - 1024 - 2 * rec - STG_BYTES - 16 - 8 * (BAR_A_FULL + 2 * 6)
    return min((free - nbb(TN, NKBB) * NKBB * b_kb) // (4 * TM * ROW_BYTES), 6)


def test_constants_match_source():
    assert "constexpr int kUmmaTM = 128, kUmmaMaxK = 256, kUmmaKB = 32;" in ENGINE
    for name, val in [("ROW_BYTES", ROW_BYTES), ("NTHREADS", NTHREADS)]:
        assert re.search(r"constexpr int %s = %d;" % (name, val), SRC), name
    assert "EPI_WARPS = 16, PROD_WARP = 16, MMA_WARP = 17" in SRC
    assert "EPI_GROUPS = EPI_WARPS / 4;" in SRC and "CHUNK_STEP = 8 * EPI_GROUPS;" in SRC
    assert "STG_BYTES = EPI_WARPS * 32 * 4 * 8;" in SRC
    assert (EPI_WARPS + 2) * 32 == NTHREADS
    # record sizes (engine.h) = the layout mirrored below
    assert "umma_a_rec_bytes(int nkb, int tm8) { return (int64_t)nkb * 256 * tm8 + kUmmaTM * 4; }" in ENGINE
    assert "umma_b_kb_bytes(int tn) { return 4 * (int64_t)tn * 64; }" in ENGINE
    assert "umma_b_rec_bytes(int nkb, int tn) { return nkb * umma_b_kb_bytes(tn) + (int64_t)tn * 4; }" in ENGINE
    assert "constexpr int kUmmaLongMaxK = 2048;" in ENGINE
    assert "static constexpr int NSTAGE = 4;" in SRC and "STAGE = umma::A_STAGE + B_KB;" in SRC


def a_tile_bytes(nkb, tm8=TM):
    return nkb * 4 * tm8 * ROW_BYTES + TM * 4


def b_tile_bytes(nkb, tn):
    return nkb * 4 * tn * ROW_BYTES + tn * 4


def layout(TN, NKBB=8):
    L = {"NSTAGE": nstage(TN, NKBB), "NKBB": NKBB, "NBB": nbb(TN, NKBB)}
    L["B_KB"] = 4 * TN * ROW_BYTES
    L["OFF_B"] = 0
    L["OFF_A"] = L["OFF_B"] + L["NBB"] * NKBB * L["B_KB"]
    L["A_PLANE"] = TM * ROW_BYTES
    L["A_STAGE"] = 4 * L["A_PLANE"]
    L["OFF_REC"] = L["OFF_A"] + L["NSTAGE"] * L["A_STAGE"]
    L["REC_EA"] = 0
    L["REC_EB"] = TM * 4
    L["REC_CB"] = L["REC_EB"] + TN * 4
    L["REC_RS"] = L["REC_CB"] + TN * 8
    L["REC_INFO"] = L["REC_RS"] + TN * 8
    L["REC_BYTES"] = L["REC_INFO"] + 16
    L["OFF_STG"] = L["OFF_REC"] + 2 * L["REC_BYTES"]
    L["OFF_BAR"] = L["OFF_STG"] + STG_BYTES
    L["NBAR"] = BAR_A_FULL + 2 * L["NSTAGE"]
    L["OFF_MISC"] = L["OFF_BAR"] + L["NBAR"] * 8
    L["BYTES"] = L["OFF_MISC"] + 16
    L["SMEM"] = L["BYTES"] + 1024
    L["TMEM_COLS"] = 8 * TN
    return L


def test_layout_formulas_match_source():
    assert "static constexpr int NSTAGE = RING_BYTES / A_STAGE < 6 ? RING_BYTES / A_STAGE : 6;" in SRC
    assert ("FREE_BYTES = 232448 - 1024 - 2 * REC_BYTES - STG_BYTES - 16 - 8 * (BAR_A_FULL + 2 * 6);") in SRC
    assert "NBB = FREE_BYTES - 2 * NKBB * B_KB >= 2 * A_STAGE ? 2 : 1;" in SRC
    assert "RING_BYTES = FREE_BYTES - NBB * NKBB * B_KB;" in SRC
    assert "BAR_B_FULL = 8," in SRC and "BAR_B_FREE = 10," in SRC and "BAR_DONE = 12," in SRC
    for TN in (16, 32, 64):
        assert [nbb(TN, k) for k in NKBBS] == {64: [1, 2, 2], 32: [2, 2, 2], 16: [2, 2, 2]}[TN]
    assert "return launch_umma_k<TN, 2>(work + ncls[0] + ncls[1], ncls[2], s, b, planes, nsm, stream);" in SRC
    assert "if (nkb > NKBB) {" in SRC
    for TN in (16, 32, 64):
        assert [nstage(TN, k) for k in NKBBS] == {64: [2, 2, 4], 32: [2, 4, 5], 16: [4, 5, 6]}[TN]
    for expr in ["B_KB = 4 * TN * ROW_BYTES", "OFF_A = OFF_B + NBB * NKBB * B_KB",
                 "OFF_REC = OFF_A + NSTAGE * A_STAGE",
                 "REC_EB = REC_EA + TM * 4", "REC_CB = REC_EB + TN * 4", "REC_RS = REC_CB + TN * 8",
                 "REC_INFO = REC_RS + TN * 8", "REC_BYTES = REC_INFO + 16", "OFF_STG = OFF_REC + 2 * REC_BYTES",
                 "OFF_BAR = OFF_STG + STG_BYTES",
                 "BAR_A_EMPTY = BAR_A_FULL + NSTAGE", "NBAR = BAR_A_FULL + 2 * NSTAGE",
                 "OFF_MISC = OFF_BAR + NBAR * 8", "BYTES = OFF_MISC + 16", "SMEM = BYTES + 1024",
                 "TMEM_COLS = 8 * TN", "A_PLANE = TM * ROW_BYTES", "A_STAGE = 4 * A_PLANE", "BAR_A_FULL = 13"]:
        assert expr in SRC, expr


@pytest.mark.parametrize("TN", [16, 32, 64])
@pytest.mark.parametrize("NKBB", NKBBS)
def test_shared_memory_regions(TN, NKBB):
    L = layout(TN, NKBB)
    assert L["SMEM"] <= SMEM_MAX
    regions = [("B", L["OFF_B"], L["OFF_A"]), ("A", L["OFF_A"], L["OFF_REC"]),
               ("rec", L["OFF_REC"], L["OFF_REC"] + 2 * L["REC_BYTES"]),
               ("stg", L["OFF_STG"], L["OFF_STG"] + STG_BYTES),
               ("bar", L["OFF_BAR"], L["OFF_BAR"] + L["NBAR"] * 8), ("misc", L["OFF_MISC"], L["OFF_MISC"] + 16)]
    assert L["OFF_STG"] % 8 == 0
    for (_, a0, a1), (_, b0, b1) in zip(regions, regions[1:]):
        assert a0 <= a1 <= b0 <= b1
    assert regions[-1][2] <= L["BYTES"]
    # base aligned to 1024 at run time: 1023 bytes of slack at most
    assert L["BYTES"] + 1023 <= L["SMEM"]
    assert L["OFF_A"] % 1024 == 0 and L["A_STAGE"] % 1024 == 0 and L["B_KB"] % 1024 == 0
    assert L["A_PLANE"] % 512 == 0 and (TN * ROW_BYTES) % 512 == 0
    # bulk-copy destinations 16-byte aligned; int64 fields 8-byte aligned
    for b in range(2):
        rec = L["OFF_REC"] + b * L["REC_BYTES"]
        assert (rec + L["REC_EA"]) % 16 == 0 and (rec + L["REC_EB"]) % 16 == 0
        assert (rec + L["REC_CB"]) % 8 == 0 and (rec + L["REC_RS"]) % 8 == 0
    assert L["OFF_BAR"] % 8 == 0
    # one CTA per SM: two would need more shared memory than an SM has, or
    # fit in TMEM together (no blocking allocation)
    assert 2 * L["SMEM"] > 228 * 1024 or 2 * L["TMEM_COLS"] <= 512
    assert L["TMEM_COLS"] in (32, 64, 128, 256, 512)


@pytest.mark.parametrize("TN", [16, 32, 64])
@pytest.mark.parametrize("nkb", [1, 2, 7, 8])
@pytest.mark.parametrize("tm8", [8, 64, 120, 128])
def test_bulk_copies(TN, nkb, tm8):
    """Every copy the producers issue: source offset inside the record, size a
    multiple of 16, destination inside its region; the bytes armed on a
    barrier phase equal the bytes copied and stay within range."""
    # the launch the planner routes an item of nkb B k blocks to
    assert "return nkb > 4 ? 0 : (nkb > 2 ? 1 : 2);" in PLANNER
    L = layout(TN, 8 if nkb > 4 else (4 if nkb > 2 else 2))
    akb = 4 * tm8 * ROW_BYTES
    A, B = a_tile_bytes(nkb, tm8), b_tile_bytes(nkb, TN)
    assert A % 16 == 0 and B % 16 == 0 and akb % 512 == 0
    # B planes of a one-pass item
    size = nkb * L["B_KB"]
    assert size % 16 == 0 and size <= L["NKBB"] * L["B_KB"] and size <= TX_MAX
    assert L["NBB"] * L["NKBB"] * L["B_KB"] == L["OFF_A"] - L["OFF_B"]
    # per row tile / pass: row exponents (end of the A record), column
    # exponents (end of the B record), the column map (TN offsets, TN strides
    # from the planner's array, 16 bytes per column)
    ea_src, eb_src = nkb * akb, nkb * L["B_KB"]
    assert ea_src % 16 == 0 and ea_src + TM * 4 == A
    assert eb_src % 16 == 0 and eb_src + TN * 4 == B
    assert L["REC_EA"] + TM * 4 == L["REC_EB"] and L["REC_EB"] + TN * 4 == L["REC_CB"]
    assert L["REC_CB"] + TN * 16 == L["REC_INFO"] and L["REC_CB"] % 16 == 0
    assert (TM * 4) % 16 == 0 and (TN * 4) % 16 == 0 and (TN * 16) % 16 == 0
    assert "bulk_g2s(rec_s + LY::REC_CB, cmaps + wk.cmap, TN * 16, bar(BAR_E_FULL + b));" in SRC
    # A k blocks into a stage (tm8-row planes, 128 rows read from each)
    assert akb <= L["A_STAGE"] and 3 * (akb // 4) + TM * ROW_BYTES <= L["A_STAGE"]
    # long kernel: one stage = A k block + B k block
    G = long_layout(TN)
    assert akb + G["B_KB"] <= TX_MAX and akb <= G["A_STAGE"]



def long_layout(TN):
    L = {"NSTAGE": 4, "A_STAGE": 4 * TM * ROW_BYTES}
    L["B_KB"] = 4 * TN * ROW_BYTES
    L["STAGE"] = L["A_STAGE"] + L["B_KB"]
    L["OFF_S"] = 0
    L["OFF_REC"] = L["NSTAGE"] * L["STAGE"]
    L["REC_BYTES"] = TM * 4 + TN * 20 + 16
    L["OFF_STG"] = L["OFF_REC"] + 2 * L["REC_BYTES"]
    L["OFF_BAR"] = L["OFF_STG"] + STG_BYTES
    L["NBAR"] = 9 + 2 * L["NSTAGE"]
    L["OFF_MISC"] = L["OFF_BAR"] + L["NBAR"] * 8
    L["BYTES"] = L["OFF_MISC"] + 16
    L["SMEM"] = L["BYTES"] + 1024
    L["TMEM_COLS"] = 8 * TN
    return L


def test_long_layout_formulas_match_source():
    for expr in ["STAGE = umma::A_STAGE + B_KB", "OFF_REC = OFF_S + NSTAGE * STAGE",
                 "OFF_STG = OFF_REC + 2 * REC_BYTES", "OFF_BAR = OFF_STG + umma::STG_BYTES",
                 "BAR_DONE = 8, BAR_S_FULL = 9, BAR_S_EMPTY = BAR_S_FULL + NSTAGE",
                 "NBAR = BAR_S_EMPTY + NSTAGE"]:
        assert expr in SRC, expr


@pytest.mark.parametrize("TN", [16, 32, 64])
def test_long_kernel_shared_memory(TN):
    L = long_layout(TN)
    assert L["SMEM"] <= SMEM_MAX and L["BYTES"] + 1023 <= L["SMEM"]
    assert L["STAGE"] % 1024 == 0 and L["B_KB"] % 1024 == 0 and L["OFF_REC"] % 16 == 0
    assert L["OFF_BAR"] % 8 == 0
    # B k block of a stage right after its 32 KB A part; the MMAs read from
    # the stage's A part (planes tm8 rows apart, 128 rows each) and B part
    for s in range(L["NSTAGE"]):
        st = s * L["STAGE"]
        for tm8 in (8, 64, 128):
            pl = tm8 * ROW_BYTES
            assert st + 3 * pl + TM * ROW_BYTES <= st + L["A_STAGE"]
        assert st + L["A_STAGE"] + 4 * TN * ROW_BYTES <= st + L["STAGE"] <= L["OFF_REC"]
    assert 2 * L["SMEM"] > 228 * 1024 or 2 * L["TMEM_COLS"] <= 512


def test_planner_plane_offsets_are_aligned():
    """Tile records are packed A tiles first, then B tiles from a 256-byte
    aligned offset: every record start is a multiple of 16."""
    import random
    rnd = random.Random(3)
    a = 0
    starts = []
    groups = [(rnd.randint(64, 3000), rnd.randint(1, 500), rnd.randint(1, 256)) for _ in range(200)]
    for M, N, K in groups:
        nkb, nrt = (K + 31) // 32, (M + 127) // 128
        for _ in range(nrt):
            starts.append(a)
            a += a_tile_bytes(nkb)
    b0 = (a + 255) // 256 * 256
    b = 0
    for M, N, K in groups:
        nkb = (K + 31) // 32
        n0 = 0
        while n0 < N:
            rem = N - n0
            tn = 64 if rem >= 64 else (16 if rem <= 16 else (32 if rem <= 32 else 64))
            starts.append(b0 + b)
            assert (2 * tn * 8) % 16 == 0   # a column map (element offsets in the map array)
            b += b_tile_bytes(nkb, tn)
            n0 += tn
    assert all(s % 16 == 0 for s in starts)


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
@pytest.mark.parametrize("NKBB", NKBBS)
def test_swizzled_stores_match_descriptor_reads(TN, NKBB):
    L = layout(TN, NKBB)
    base = 1024 * 7   # any 1024-aligned dynamic-smem base
    # A: record k block kb (planes tm8 rows apart) -> stage s; plane p, row
    # r < tm8, slot j (the prepare kernel's cut8_store(row=r) into a plane of
    # tm8 * 64 bytes)
    for tm8 in (8, 56, 128):
        pl = tm8 * ROW_BYTES
        for s in range(L["NSTAGE"]):
            for kb in (0, 3):
                for p in range(4):
                    for r in range(tm8):
                        for j in range(KB_SLOTS):
                            rec_off = kb * 4 * pl + p * pl + store_offset(r, j // 8) + (j % 8) * 2
                            # the bulk copy moves k block kb's bytes unchanged to the stage
                            w = base + L["OFF_A"] + s * L["A_STAGE"] + (rec_off - kb * 4 * pl)
                            plane = base + L["OFF_A"] + s * L["A_STAGE"] + p * pl
                            k16, k = divmod(j, 16)
                            assert tensor_core_read(plane + k16 * 32, r, k) == w
                            assert plane <= w < plane + pl
    # B': record k block kb, plane p, column c -> operand row p*TN + c; the
    # whole record's planes are copied to B buffer bb (at most NKBB k blocks)
    assert "bulk_g2s(base_s + LY::OFF_B + bb * (NKBB * LY::B_KB), brec, (uint32_t)(nkb * LY::B_KB)," in SRC
    assert "const uint32_t b_s = base_s + LY::OFF_B + bb * (NKBB * LY::B_KB) + kb * LY::B_KB;" in SRC
    for bb, kb in [(bb, kb) for bb in range(L["NBB"]) for kb in range(NKBB)]:
        blk = base + L["OFF_B"] + bb * NKBB * L["B_KB"] + kb * L["B_KB"]
        for p in range(4):
            for c in range(TN):
                for j in range(KB_SLOTS):
                    rec_off = kb * L["B_KB"] + p * TN * ROW_BYTES + store_offset(c, j // 8) + (j % 8) * 2
                    w = base + L["OFF_B"] + bb * NKBB * L["B_KB"] + rec_off
                    k16, k = divmod(j, 16)
                    assert tensor_core_read(blk + k16 * 32, p * TN + c, k) == w
                    assert blk <= w < blk + L["B_KB"] and w < base + L["OFF_A"]


@pytest.mark.parametrize("TN", [16, 32, 64])
@pytest.mark.parametrize("NKBB", NKBBS)
def test_mma_operand_and_tmem_ranges(TN, NKBB):
    L = layout(TN, NKBB)
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


def test_epilogue_staging_and_tmem_chunks():
    """Epilogue warp w: TMEM lane quarter w % 4, 8-column chunks from 8 (w / 4)
    in steps of 32 (at most NCH per warp, the long kernel's register sums);
    its 1 KB staging area holds 32 rows x 4 float64 (a chunk is stored in two
    halves); the swizzled writes (lane = row) and reads (8 rows x 4 columns
    per instruction) cover the area exactly once each, without bank
    conflicts."""
    assert "tcgen05.ld.sync.aligned.32x32b.x8.b32" in SRC
    assert SRC.count("const int quarter = warp & 3, group = warp >> 2;") == 2
    assert "for (int c0 = 8 * group; c0 < TN; c0 += CHUNK_STEP) {" in SRC
    assert SRC.count("const int c0 = 8 * group + CHUNK_STEP * jc;") == 2
    assert "constexpr int NCH = (TN / 8 + EPI_GROUPS - 1) / EPI_GROUPS;" in SRC
    assert SRC.count("double *stg = reinterpret_cast<double *>(sm + LY::OFF_STG) + warp * 128;") == 2
    assert EPI_WARPS % 4 == 0
    groups = EPI_WARPS // 4
    for TN in (16, 32, 64):
        cover = {}
        nch = (TN // 8 + groups - 1) // groups
        for w in range(EPI_WARPS):
            q, h = w & 3, w >> 2
            assert len(range(8 * h, TN, 8 * groups)) <= nch
            for c0 in range(8 * h, TN, 8 * groups):
                for lane in range(32):
                    for i in range(8):
                        key = (q * 32 + lane, c0 + i)
                        cover[key] = cover.get(key, 0) + 1
        assert len(cover) == TM * TN and set(cover.values()) == {1}
    widx = lambda lane, i: lane * 4 + (i ^ ((lane >> 2) & 3))
    ridx = lambda r, col: r * 4 + (col ^ ((r >> 2) & 3))
    assert "stg[lane * 4 + (i ^ ((lane >> 2) & 3))] = val[4 * h + i];" in SRC
    assert "stg[r * 4 + (col ^ ((r >> 2) & 3))];" in SRC
    assert "const int r = k * 8 + (lane >> 2);" in SRC
    writes = sorted(widx(lane, i) for lane in range(32) for i in range(4))
    reads = sorted(ridx(k * 8 + (lane >> 2), lane & 3) for k in range(4) for lane in range(32))
    assert writes == list(range(128)) and reads == list(range(128))
    # a read instruction: 8 rows x 4 columns, 8 distinct rows, all 4 columns each
    for k in range(4):
        assert len({k * 8 + (lane >> 2) for lane in range(32)}) == 8
    # no bank conflicts: an 8-byte access is served per half warp (128 bytes);
    # its 16 lanes must hit 16 different bank pairs
    for hw in (range(0, 16), range(16, 32)):
        for i in range(4):
            assert len({widx(lane, i) % 16 for lane in hw}) == 16
        for k in range(4):
            assert len({ridx(k * 8 + (lane >> 2), lane & 3) % 16 for lane in hw}) == 16


def test_prepare_a_thread_maps():
    """k_prep_a: for every block shape (W = the window's slots rounded up to a
    power of two, RB = 4096 / W rows), the 256 threads' 16 loads cover every
    (row, slot) of the block once in both load maps (along the rows of a
    slot, along the slots of a row), stay inside the staging buffer, the
    exponent map gives each row 256 / RB threads, and the cut map covers every
    (k block, row, chunk) of the block once."""
    assert "constexpr int PREP_ELEMS = 4096;" in SRC and "constexpr int PREP_STAGE = 128 * (32 + 2);" in SRC
    assert "const int lw = nkb <= 1 ? 5 : (nkb <= 2 ? 6 : (nkb <= 4 ? 7 : 8));  // log2 W" in SRC
    assert "const int W = 1 << lw, lrb = 12 - lw, RB = 1 << lrb, pitch = W + 2;" in SRC
    assert "const int t_r = rows_fast ? (tid & (RB - 1)) : (tid >> lw);" in SRC
    assert "const int t_j = rows_fast ? (tid >> lrb) : (tid & (W - 1));" in SRC
    assert "const int step = rows_fast ? (PREP_THREADS >> lrb) : (PREP_THREADS >> lw);" in SRC
    assert "const int ch = u & 3, r = (u >> 2) & (RB - 1), kb = u >> (lrb + 2);" in SRC
    assert "const int ltpr = 8 - lrb, tpr = 1 << ltpr;" in SRC
    STAGE = 128 * 34
    for nkb in range(1, KMAX // KB_SLOTS + 1):
        lw = 5 if nkb <= 1 else (6 if nkb <= 2 else (7 if nkb <= 4 else 8))
        W, lrb = 1 << lw, 12 - lw
        RB, pitch = 1 << lrb, W + 2
        assert nkb * KB_SLOTS <= W and RB * pitch <= STAGE
        for rows_fast in (True, False):
            seen = set()
            for tid in range(256):
                t_r = (tid & (RB - 1)) if rows_fast else (tid >> lw)
                t_j = (tid >> lrb) if rows_fast else (tid & (W - 1))
                step = (256 >> lrb) if rows_fast else (256 >> lw)
                for i in range(16):
                    r = t_r if rows_fast else t_r + step * i
                    j = t_j + step * i if rows_fast else t_j
                    assert 0 <= r < RB and 0 <= j < W and r * pitch + j < STAGE
                    seen.add((r, j))
            assert len(seen) == RB * W
        tpr = 256 // RB
        assert {tid >> (8 - lrb) for tid in range(256)} == set(range(RB)) and 32 % tpr == 0
        cut = [(u >> (lrb + 2), (u >> 2) & (RB - 1), u & 3) for u in range(nkb << (lrb + 2))]
        assert len(set(cut)) == len(cut) == nkb * RB * 4
        assert all(kb < nkb and kb * KB_SLOTS + ch * 8 + 7 < W for kb, r, ch in cut)
