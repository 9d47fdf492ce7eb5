"""Index arithmetic of the tcgen05 GEMM (rewl_simulator_gb300/csrc/mlp.cu, k_gemm_tc) restated
and checked on the CPU: every copy mapping fills each byte of its shared stage exactly once and
stays inside it, and the four MMAs of a K block, walking their shared-memory descriptors
(start + 8-row group x SBO + K core matrix x LBO, 8 rows of 16 B per core matrix), read exactly
the elements the copies wrote, in (row, k) order."""
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
LBO, SBO = _const("kLBO"), _const("kSBO")


def core_off(r, k):
    return (r >> 3) * SBO + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2


def copy_map(R, kmaj):
    """(row, k) -> byte offset written by issue_tile<R, KMAJ>, over all 128 threads."""
    out = {}
    for tid in range(128):
        for c in range(tid, R * (BK // 8), 128):
            if kmaj:
                r, kq = (c & 7) | ((c >> 6) << 3), (c >> 3) & 7
                cells = [((r, kq * 8 + i), core_off(r, kq * 8) + 2 * i) for i in range(8)]
            else:
                mg, k = c % (R // 8), c // (R // 8)
                base = mg * SBO + (k >> 3) * LBO + (k & 7) * 16
                cells = [((mg * 8 + i, k), base + 2 * i) for i in range(8)]
            for key, off in cells:
                assert key not in out
                out[key] = off
    return out


def mma_reads(R, kmaj, kk):
    """(row, k) -> byte offset read by MMA kk (K 16) from a descriptor at start kk * 2 * LBO."""
    start, out = kk * 2 * LBO, {}
    for r in range(R):
        for kc in range(2):
            for j in range(8):
                k = kk * 16 + kc * 8 + j
                if kmaj:     # core row = 8 consecutive k of one row
                    off = start + (r >> 3) * SBO + kc * LBO + (r & 7) * 16 + j * 2
                else:        # core row = 8 consecutive rows at one k
                    off = start + (r >> 3) * SBO + kc * LBO + j * 16 + (r & 7) * 2
                out[(r, k)] = off
    return out


@pytest.mark.parametrize("R", [BM, BN])
@pytest.mark.parametrize("kmaj", [True, False])
def test_copies_fill_the_stage_once(R, kmaj):
    m = copy_map(R, kmaj)
    assert set(m) == {(r, k) for r in range(R) for k in range(BK)}
    offs = np.array(sorted(m.values()))
    assert offs[0] == 0 and offs[-1] == R * BK * 2 - 2
    assert np.array_equal(offs, np.arange(0, R * BK * 2, 2))


@pytest.mark.parametrize("R", [BM, BN])
@pytest.mark.parametrize("kmaj", [True, False])
def test_mma_descriptors_read_what_the_copies_wrote(R, kmaj):
    written = copy_map(R, kmaj)
    for kk in range(BK // 16):
        for key, off in mma_reads(R, kmaj, kk).items():
            assert written[key] == off, (kk, key)


def test_instruction_descriptor_fields():
    # kind::f16: D FP32, A/B BF16, transpose bits 15/16, N >> 3 at bit 17, M >> 4 at bit 24
    def idesc(a_mn, b_mn):
        return (1 << 4) | (1 << 7) | (1 << 10) | (a_mn << 15) | (b_mn << 16) | ((BN >> 3) << 17) | ((BM >> 4) << 24)
    assert idesc(0, 0) == 0x08100490
    assert (idesc(0, 0) >> 17) & 0x3F == BN // 8 and (idesc(0, 0) >> 24) & 0x1F == BM // 16
    assert "((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16)" in SRC
    assert BM == 128 and BN % 16 == 0 and 16 <= BN <= 256
