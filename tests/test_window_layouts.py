"""The row tile's shared-memory window layouts, restated from matx_gb300/csrc/rowtile.cuh
(smem_idx, unit_idx): each is a permutation inside its block, and the row-strided reads of a
warp hit distinct banks.  Lanes read rows q*S + k of the window: 8-byte loads are served per
half-warp (16 lanes, 16 slots of 8 bytes per 128-byte wavefront), 4-byte loads of real
samples per warp (32 lanes, 32 banks), the paired form's 16-byte loads per quarter-warp (8
lanes, 8 units of 16 bytes)."""
import pytest


def ctz(v):
    t = 0
    while v and not (v >> t) & 1:
        t += 1
    return t


def smem_idx(p, pad):
    """Element XOR layout for an even row stride S, pad = 10 + ctz(S)."""
    t = pad - 10
    sh, m = max(t, 4), (1 << min(t, 4)) - 1
    return p ^ ((p >> sh) & m)


def smem_idx_real(p, pad):
    """Element XOR layout of real float samples for an even row stride S, pad = 30 + ctz(S)."""
    t = pad - 30
    sh, m = max(t, 5), (1 << min(t, 5)) - 1
    return p ^ ((p >> sh) & m)


def unit_idx(u, pad):
    """Unit (two complex samples) layout of the paired walk, pad = 20 + ctz(S/2)."""
    if pad == 20:
        return u
    t = pad - 20
    sh, m = max(t, 3), (1 << min(t, 3)) - 1
    return u ^ ((u >> sh) & m)


@pytest.mark.parametrize("pad", list(range(11, 18)))
def test_element_layout_is_a_block_permutation(pad):
    for base in (0, 16, 4096):
        block = [smem_idx(base + i, pad) for i in range(16)]
        assert sorted(block) == list(range(base, base + 16))


@pytest.mark.parametrize("pad", list(range(20, 28)))
def test_unit_layout_is_a_block_permutation(pad):
    for base in (0, 8, 4096):
        block = [unit_idx(base + i, pad) for i in range(8)]
        assert sorted(block) == list(range(base, base + 8))


def test_element_layout_conflict_free():
    for S in range(2, 256, 2):
        pad = 10 + ctz(S)
        if pad > 17:
            continue
        for c in range(64):
            for h in (0, 16):
                slots = {smem_idx(c + (h + lane) * S, pad) % 16 for lane in range(16)}
                assert len(slots) == 16, (S, c, h)


def test_unit_layout_conflict_free():
    for s2 in range(1, 256):
        t = ctz(s2)
        if t > 7:
            continue
        pad = 20 + t
        for c in range(64):
            for q in range(0, 32, 8):
                slots = {unit_idx(c + (q + lane) * s2, pad) % 8 for lane in range(8)}
                assert len(slots) == 8, (s2, c, q)


@pytest.mark.parametrize("pad", list(range(31, 38)))
def test_real_layout_is_a_block_permutation(pad):
    for base in (0, 32, 8192):
        block = [smem_idx_real(base + i, pad) for i in range(32)]
        assert sorted(block) == list(range(base, base + 32))


def test_real_layout_conflict_free():
    for S in range(2, 256, 2):
        pad = 30 + min(ctz(S), 7)
        for c in range(64):
            banks = {smem_idx_real(c + lane * S, pad) % 32 for lane in range(32)}
            assert len(banks) == 32, (S, c)
