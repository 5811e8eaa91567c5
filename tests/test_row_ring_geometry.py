"""The row ring's copy geometry (the FP32 step kernels' prefetch level 3).

A restatement in Python of the index arithmetic march_strip uses with its
row ring (swm_gb300/csrc/march.cu: the `issue` copies, `ridx` reads, and the
RING_* sizes), checked for every strip of many basin widths and for rows
that wrap around the periodic boundary in j.  Checked here:

- every bulk copy starts on a 16-byte boundary and moves a whole number of
  16-byte words;
- no copy reads more than 16 bytes past its field, the padding the
  allocations leave;
- the two pieces of a field fit its slot region without overlapping;
- every lane reads its own column's element at an index inside its region.

Runs on the CPU: it guards the kernel's addresses before any GPU run.
"""
import random

import pytest

RING_FB, RING_MB, RING_NF = 192, 128, 13
RING_MIN_NX = 32


def _wrapm(g, n):
    g = g + n if g < 0 else g
    return g - n if g >= n else g


def _strip(nx, ny, H, bx, rows):
    TI = 32 - 2 * H
    gx0 = bx * TI - H
    am = max(gx0, 0)
    wm = min(gx0 + 32, nx) - am
    aw = gx0 + nx if gx0 < 0 else 0
    ww = -gx0 if gx0 < 0 else max(gx0 + 32 - nx, 0)
    assert wm > 0 and wm + ww == 32
    for Jr in rows:
        r = nx * _wrapm(Jr, ny)
        slot = {}  # field -> {slot element: global element}
        for lane in range(28):
            fi, pc = lane >> 1, lane & 1
            pa, pw = (aw, ww) if pc else (am, wm)
            if pw <= 0:
                continue
            fes, fal = (2, 7) if fi == 13 else (4, 3)
            s0 = (r + pa) & fal
            nel = (s0 + pw + fal) & ~fal
            before = ((((r + am) & fal) + wm + fal) & ~fal) if pc else 0
            start = r + pa - s0
            assert (start * fes) % 16 == 0 and (nel * fes) % 16 == 0 and nel > 0
            assert (start + nel) * fes <= nx * ny * fes + 16
            assert before * fes + nel * fes <= (RING_MB if fi == 13 else RING_FB)
            d = slot.setdefault(fi, {})
            for k in range(nel):
                assert before + k not in d  # the pieces do not overlap
                d[before + k] = start + k
        for lane in range(32):
            gx = gx0 + lane
            gi = gx % nx
            inw = gx < 0 or gx >= nx
            lofs = gi - (aw if inw else am)
            for fi, al in ((0, 3), (7, 3), (13, 7)):
                s0 = (r + am) & al
                idx = (((s0 + wm + al) & ~al) + ((r + aw) & al) + lofs) if inw else s0 + lofs
                assert 0 <= idx < ((RING_MB // 2) if fi == 13 else RING_FB // 4)
                assert slot[fi][idx] == r + gi, (nx, bx, lane, fi)


@pytest.mark.parametrize('H', [1, 2])
def test_row_ring_copies_and_reads(H):
    rnd = random.Random(7 + H)
    widths = list(range(RING_MIN_NX, 140)) + [255, 256, 257, 511, 512, 513, 1023, 1025, 2049]
    TI = 32 - 2 * H
    for nx in widths:
        ny = rnd.choice([5, 17, 64, 100, 1025])
        rows = list(range(-3, min(ny, 8))) + [ny - 1, ny, ny + 1] + rnd.sample(range(ny), min(ny, 3))
        for bx in range((nx + TI - 1) // TI):
            _strip(nx, ny, H, bx, rows)


def test_slot_sizes_match_the_kernel():
    """The constants above are those of march.cu."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            'swm_gb300', 'csrc', 'march.cu')).read()
    for name, val in (('RING_FB', RING_FB), ('RING_MB', RING_MB), ('RING_NF', RING_NF)):
        m = re.search(r'constexpr int %s = (\d+);' % name, src)
        assert m and int(m.group(1)) == val, name
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            'swm_gb300', 'csrc', 'fused32.h')).read()
    m = re.search(r'constexpr int RING_MIN_NX = (\d+);', hdr)
    assert m and int(m.group(1)) == RING_MIN_NX
