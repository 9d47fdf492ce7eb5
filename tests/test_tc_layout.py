"""Index arithmetic of the tcgen05 GEMM (rewl_simulator_gb300/csrc/mlp.cu, k_gemm_tc) restated
and checked on the CPU: the tensor-memory-accelerator boxes of a stage (load_tile) fill each byte
of their shared tile exactly once and stay inside it, every box starts on a 16-byte column and a
1024-byte-aligned shared address, and the four MMAs of a K block, walking their shared-memory
descriptors (tile_desc: start + 8-row group x SBO + K core matrix x LBO, 8 rows of 16 B per core
matrix), read exactly the elements the boxes wrote, in (row, k) order."""
import re

import numpy as np
import pytest

from conftest import ROOT

SRC = (ROOT / "rewl_simulator_gb300" / "csrc" / "mlp.cu").read_text()


def _const(name):
    m = re.search(rf"constexpr (?:int|uint32_t) {name} = (\d+)", SRC) or \
        re.search(rf"constexpr int [^;]*\b{name} = (\d+)", SRC)
    assert m, name
    return int(m.group(1))


BM, BN, BK = _const("BM"), _const("BN"), _const("BK")


def boxes(R, kmaj):
    """(shared offset, x, y, box inner, box outer) of each box load_tile<R, KMAJ> issues for the
    tile at rows 0.., k 0.. (x along the contiguous dimension)."""
    if kmaj:     # boxes of 8 k x R rows, one per 8-wide column of k, R x 16 B apart
        return [(c * R * 16, 8 * c, 0, 8, R) for c in range(BK // 8)]
    return [(g * 1024, 8 * g, 0, 8, BK) for g in range(R // 8)]   # 8 rows x BK k, 1024 B apart


def box_map(R, kmaj):
    """(row, k) -> byte offset written by the boxes (a box lands row-major: inner 16 B rows)."""
    out = {}
    for off, x, y, inner, outer in boxes(R, kmaj):
        for o in range(outer):
            for i in range(inner):
                key = (y + o, x + i) if kmaj else (x + i, y + o)      # (row, k)
                assert key not in out
                out[key] = off + o * inner * 2 + i * 2
    return out


def mma_reads(R, kmaj, kk):
    """(row, k) -> byte offset read by MMA kk (K 16) through tile_desc<R, KMAJ>(0, kk)."""
    if kmaj:
        start, lbo, sbo = kk * 2 * R * 16, R * 16, 128
    else:
        start, lbo, sbo = kk * 256, 128, 1024
    out = {}
    for r in range(R):
        for kc in range(2):
            for j in range(8):
                k = kk * 16 + kc * 8 + j
                if kmaj:     # core row = 8 consecutive k of one row
                    off = start + (r >> 3) * sbo + kc * lbo + (r & 7) * 16 + j * 2
                else:        # core row = 8 consecutive rows at one k
                    off = start + (r >> 3) * sbo + kc * lbo + j * 16 + (r & 7) * 2
                out[(r, k)] = off
    return out


@pytest.mark.parametrize("R", [BM, BN])
@pytest.mark.parametrize("kmaj", [True, False])
def test_boxes_fill_the_tile_once(R, kmaj):
    m = box_map(R, kmaj)
    assert set(m) == {(r, k) for r in range(R) for k in range(BK)}
    offs = np.array(sorted(m.values()))
    assert np.array_equal(offs, np.arange(0, R * BK * 2, 2))
    for off, x, _, inner, outer in boxes(R, kmaj):
        assert (x * 2) % 16 == 0 and inner * 2 == 16           # 16-byte column, 16-byte box rows
        assert off % 1024 == 0 and inner * outer * 2 <= 2048


@pytest.mark.parametrize("R", [BM, BN])
@pytest.mark.parametrize("kmaj", [True, False])
def test_mma_descriptors_read_what_the_boxes_wrote(R, kmaj):
    written = box_map(R, kmaj)
    for kk in range(BK // 16):
        for key, off in mma_reads(R, kmaj, kk).items():
            assert written[key] == off, (kk, key)


def test_source_layout_matches_this_restatement():
    assert "tma_load_2d(dst + c * (R * 16), map, k0 + 8 * c, r0, bar)" in SRC
    assert "tma_load_2d(dst + g * 1024, map, r0 + 8 * g, k0, bar)" in SRC
    assert "smem_desc(addr + kk * 2 * (R * 16), R * 16, 128) : smem_desc(addr + kk * 256, 128, 1024)" in SRC
    assert "const cuuint32_t box[2] = {8, (cuuint32_t)box_outer};" in SRC
    # stage bytes armed on the full barrier = the boxes' bytes
    assert BM * BK * 2 + BN * BK * 2 == sum(i * o * 2 for _, _, _, i, o in boxes(BM, True) + boxes(BN, True))


def test_instruction_descriptor_fields():
    # kind::f16: D FP32, A/B BF16, transpose bits 15/16, N >> 3 at bit 17, M >> 4 at bit 24
    def idesc(a_mn, b_mn):
        return (1 << 4) | (1 << 7) | (1 << 10) | (a_mn << 15) | (b_mn << 16) | ((BN >> 3) << 17) | ((BM >> 4) << 24)
    assert idesc(0, 0) == 0x08100490
    assert (idesc(0, 0) >> 17) & 0x3F == BN // 8 and (idesc(0, 0) >> 24) & 0x1F == BM // 16
    assert "((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16)" in SRC
    assert BM == 128 and BN % 16 == 0 and 16 <= BN <= 256
