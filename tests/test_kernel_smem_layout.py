"""Shared-memory layout of the tensor-core kernels, checked on the CPU.

Every shared-memory address the split kernels form (digit-plane stores of the
cut, ldmatrix row addresses of the products, exponents, slot tables, the
control words) is recomputed here for every template instance and every
thread, and checked against its region, its alignment and the 227 KB limit.
The constants mirror csrc/kernels.cu; the source lines they come from are
asserted verbatim first, so a change of the kernel's tiling fails here until
the mirror is updated.
"""
import os

import pytest

SRC = os.path.join(os.path.dirname(__file__), "..", "zmpo_dmrg_gb300", "csrc", "kernels.cu")
COMMON = os.path.join(os.path.dirname(__file__), "..", "zmpo_dmrg_gb300", "csrc", "device_common.cuh")
SLOT = 56              # sizeof(Slot): 2 pointers, 2 int64, 1 double, 4 int
LIMIT = 232448         # dynamic + static shared memory per CTA
NPART = 4              # independent parts of a B-resident CTA

MIRRORED = [
    "static constexpr int TK = (S == 4 && TN == 64) ? 64 : 32;",
    "static constexpr int PAD = TK + 8;",
    "static constexpr int NCH = 8;",
    "static constexpr int WM = TM / 16, WN = TN / 8;",
    "static constexpr int NT = 32 * WM * WN;",
    "static constexpr int TPR = NT / TM;",
    "static constexpr int KPA = TK / TPR;",
    "static constexpr int TPC = NT / TN;",
    "static constexpr int KPB = TK / TPC;",
    "static constexpr int CHB = 256 / Sh::TK;",
    "static constexpr int EBN = TN < 16 ? 16 : TN;",
    "constexpr int NPART = 4;",
    "constexpr int TMH = TM / NPART, NTH = Sh::NT / NPART, WMH = TMH / 16;",
    "constexpr int TPRH = NTH / TMH, KPAH = TK / TPRH;",
    "(size_t)CHB * EBN * 4 + (size_t)CHB * Sh::TK * sizeof(Slot) + (4 + CHB) * 4 + 16;",
    "(4 + Sh::NCH) * sizeof(int) + 16;",
]
# the slot record lives in the header both kernel files include
MIRRORED_COMMON = ["int pad;\n};"]


def test_mirrored_constants_match_the_kernel_source():
    src = open(SRC).read()
    for line in MIRRORED:
        assert line in src, "kernels.cu changed: update this mirror (%s)" % line
    common = open(COMMON).read()
    for line in MIRRORED_COMMON:
        assert line in common, "device_common.cuh changed: update this mirror (%s)" % line


def shape(S, TM, TN):
    TK = 64 if (S == 4 and TN == 64) else 32
    WM, WN = TM // 16, TN // 8
    NT = 32 * WM * WN
    TPR, TPC = NT // TM, NT // TN
    return dict(TK=TK, PAD=TK + 8, NCH=8, WM=WM, WN=WN, NT=NT, TPR=TPR, KPA=TK // TPR, TPC=TPC,
                KPB=TK // TPC, EBN=max(TN, 16))


def check_cut(S, rows, T, K, PAD, plane0, plane1, row, part, per_thread):
    """Digit-plane stores of one thread's slots (row, slots part*per .. +per)."""
    for s in range(S):
        for t in range(per_thread):
            col = part * per_thread + t
            assert col < K
            off = plane0 + ((s * rows + row) * PAD + col) * 2
            assert plane0 <= off and off + 2 <= plane1
        if S == 4 and per_thread % 2 == 0:  # packed pairs: 4-byte stores
            assert ((row * PAD + part * per_thread) * 2) % 4 == 0


def check_ldmatrix(S, lane, wm, wn, TMp, TN, TK, PAD, A0, A1, B0, B1):
    a_base = A0 + ((wm + (lane & 7) + ((lane >> 3) & 1) * 8) * PAD + (lane >> 4) * 8) * 2
    b_base = B0 + (((lane >> 4) * TN + wn + (lane & 7)) * PAD + ((lane >> 3) & 1) * 8) * 2
    for kk in range(0, TK, 16):
        for sa in range(S):
            addr = a_base + sa * TMp * PAD * 2 + kk * 2
            assert addr % 16 == 0 and A0 <= addr and addr + 16 <= A1
        for sb in range(0, S - 1, 2):
            addr = b_base + sb * TN * PAD * 2 + kk * 2
            assert addr % 16 == 0 and addr + 16 <= B1
        if S % 2 == 1 and lane < 16:
            addr = b_base + (S - 1) * TN * PAD * 2 + kk * 2
            assert addr % 16 == 0 and addr + 16 <= B1


TILES = [(S, TM, TN) for S in (4, 7) for TM in (32, 64, 128) for TN in (8, 16, 32, 64)
         if not (TN == 64 and TM == 128)]


@pytest.mark.parametrize("S,TM,TN", TILES)
def test_tile_kernel_shared_memory(S, TM, TN):
    c = shape(S, TM, TN)
    TK, PAD, NCH, NT, EBN = c["TK"], c["PAD"], c["NCH"], c["NT"], c["EBN"]
    assert NT <= 1024 and min(c["TPR"], c["KPA"], c["TPC"], c["KPB"]) >= 1
    Ap0, Ap1 = 0, S * TM * PAD * 2
    Bp0, Bp1 = Ap1, Ap1 + S * TN * PAD * 2
    Ea0, Ea1 = Bp1, Bp1 + TM * 4
    Eb0, Eb1 = Ea1, Ea1 + EBN * 4
    Sl0, Sl1 = Eb1, Eb1 + NCH * TK * SLOT
    ct0, ct1 = Sl1, Sl1 + (4 + NCH) * 4
    smem = S * (TM + TN) * PAD * 2 + (TM + EBN) * 4 + NCH * TK * SLOT + (4 + NCH) * 4 + 16
    assert ct1 <= smem and smem + 2 * TN * 4 <= LIMIT
    assert Bp0 % 16 == 0 and Sl0 % 8 == 0
    for tid in range(NT):
        lane, warp = tid & 31, tid >> 5
        wm, wn = (warp % c["WM"]) * 16, (warp // c["WM"]) * 8
        ra, parta = tid // c["TPR"], tid % c["TPR"]
        cb, partb = tid // c["TPC"], tid % c["TPC"]
        assert ra < TM and cb < TN and Ea0 + ra * 4 + 4 <= Ea1 and Eb0 + cb * 4 + 4 <= Eb1
        check_cut(S, TM, NT, TK, PAD, Ap0, Ap1, ra, parta, c["KPA"])
        check_cut(S, TN, NT, TK, PAD, Bp0, Bp1, cb, partb, c["KPB"])
        assert wm + 16 <= TM and wn + 8 <= TN
        check_ldmatrix(S, lane, wm, wn, TM, TN, TK, PAD, Ap0, Ap1, Bp0, Bp1)
    # the slot table of a pass and the control words (cursor, nchunk, nslot, scaled)
    assert Sl0 + NCH * TK * SLOT <= Sl1 and ct0 + (3 + NCH) * 4 + 4 <= ct1


@pytest.mark.parametrize("TM,TN", [(64, 64), (128, 32)])
def test_b_resident_kernel_shared_memory(TM, TN):
    S = 4
    c = shape(S, TM, TN)
    TK, PAD, NT, EBN = c["TK"], c["PAD"], c["NT"], c["EBN"]
    CHB = 256 // TK
    TMH, NTH = TM // NPART, NT // NPART
    WMH, TPRH = TMH // 16, NTH // TMH
    KPAH = TK // TPRH
    assert WMH * c["WN"] * 32 == NTH and TPRH * KPAH == TK and 32 % TPRH == 0
    BPL = S * TN * PAD
    Ap0, Ap1 = 0, S * TM * PAD * 2
    Bp0, Bp1 = Ap1, Ap1 + CHB * BPL * 2
    Ea0, Ea1 = Bp1, Bp1 + TM * 4
    Eb0, Eb1 = Ea1, Ea1 + CHB * EBN * 4
    Sl0, Sl1 = Eb1, Eb1 + CHB * TK * SLOT
    ct0, ct1 = Sl1, Sl1 + (4 + CHB) * 4
    smem = (4 * TM * PAD * 2 + CHB * 4 * TN * PAD * 2 + TM * 4 + CHB * EBN * 4 + CHB * TK * SLOT
            + (4 + CHB) * 4 + 16)
    assert ct1 <= smem and smem + 2 * TN * 4 <= LIMIT and Sl0 % 8 == 0
    for tid in range(NT):
        lane, warp = tid & 31, tid >> 5
        part, tidh = tid // NTH, tid % NTH
        assert (tid - lane) // NTH == part  # a warp lies in one part (named barriers)
        warph = tidh >> 5
        wm, wn = (warph % WMH) * 16, (warph // WMH) * 8
        ra, parta = tidh // TPRH, tidh % TPRH
        cb, partb = tid // c["TPC"], tid % c["TPC"]
        Aph0 = Ap0 + part * S * TMH * PAD * 2
        Aph1 = Aph0 + S * TMH * PAD * 2
        assert ra < TMH and Ea0 + (part * TMH + ra) * 4 + 4 <= Ea0 + (part + 1) * TMH * 4 <= Ea1
        check_cut(S, TMH, NTH, TK, PAD, Aph0, Aph1, ra, parta, KPAH)
        assert wm + 16 <= TMH and wn + 8 <= TN
        for ch in range(CHB):
            Bc0 = Bp0 + ch * BPL * 2
            assert Eb0 + (ch * EBN + cb) * 4 + 4 <= Eb1
            check_cut(S, TN, NT, TK, PAD, Bc0, Bc0 + BPL * 2, cb, partb, c["KPB"])
            check_ldmatrix(S, lane, wm, wn, TMH, TN, TK, PAD, Aph0, Aph1, Bc0, Bc0 + BPL * 2)
    assert Sl0 + CHB * TK * SLOT <= Sl1 and ct0 + (3 + CHB) * 4 + 4 <= ct1
