"""The planner of the FP32 step kernel's tiles (swm_gpu_plan_step_tiles),
host code only, run here without a GPU.

The kernel updates each (strip, row) exactly once, from the tile that holds
it; the GPU tests check that results do not depend on the tiles.  Here: every
row of every strip lies in exactly one tile, tiles come four to a block with
padding only at the end, equal costs give equal groups, and rows whose
window holds land (the coastal strips) get shorter groups as their cost
rises."""
import ctypes
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def L():
    from swm_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from swm_gb300 import build
        build.build()
    return _lib.lib()


def mask_words(ocean_e):
    """Packed mask words as the fused set-up builds them, from an eta-point
    ocean mask (ny, nx): u, v and H points are ocean where the cells they
    join are (a simplified closed-basin rule); bits 4-7 and 8-11 hold the
    i-1 and i+1 neighbours' bits, periodic in i."""
    e = ocean_e.astype(np.uint16)
    u = e & np.roll(e, 1, axis=1)
    v = e & np.roll(e, 1, axis=0)
    h = u & np.roll(u, 1, axis=0)
    own = h | (u << 1) | (v << 2) | (e << 3)
    return (own | (np.roll(own, 1, axis=1) << 4) | (np.roll(own, -1, axis=1) << 8)).astype(np.uint16)


def plan(L, mix, m16, rows, cost):
    ny, nx = m16.shape
    m = np.ascontiguousarray(m16)
    n = L.swm_gpu_plan_step_tiles(mix, nx, ny, m.ctypes.data_as(ctypes.c_void_p), rows, cost, None, 0)
    assert n > 0 and n % 4 == 0
    out = np.zeros((n, 3), dtype=np.int32)
    assert L.swm_gpu_plan_step_tiles(mix, nx, ny, m.ctypes.data_as(ctypes.c_void_p), rows, cost,
                                     out.ctypes.data_as(ctypes.c_void_p), n) == n
    return out


def strips_of(mix, nx):
    from swm_gb300 import _lib
    cols = _lib.lib().swm_gpu_step_strip_columns(mix)
    assert cols in (32 - 2 * (2 if mix == 2 else 1), 64 - 2 * (2 if mix == 2 else 1))
    return (nx + cols - 1) // cols


def basins():
    rng = np.random.Generator(np.random.PCG64(7))
    box = np.ones((70, 90), bool)
    box[0, :] = box[-1, :] = box[:, 0] = box[:, -1] = False
    islands = box.copy()
    for _ in range(12):
        j, i = rng.integers(2, 68), rng.integers(2, 88)
        islands[j - 1:j + 2, i - 1:i + 2] = False
    return {'box': box, 'islands': islands, 'ocean': np.ones((40, 61), bool), 'narrow': box[:, :7].copy()}


@pytest.mark.parametrize('mix', [0, 1, 2])
@pytest.mark.parametrize('name', ['box', 'islands', 'ocean', 'narrow'])
@pytest.mark.parametrize('rows,cost', [(4, 1.0), (16, 1.0), (17.25, 1.7), (32, 2.6), (250, 1.0)])
def test_every_row_of_every_strip_once(L, mix, name, rows, cost):
    m16 = mask_words(basins()[name])
    ny, nx = m16.shape
    t = plan(L, mix, m16, rows, cost)
    busy = t[:, 2] > 0
    # padding only in the last block
    assert busy[:len(t) - 3].all()
    cover = np.zeros((strips_of(mix, nx), ny), int)
    for s, r0, k in t[busy]:
        assert 0 <= s < cover.shape[0] and 1 <= k <= 255 and r0 + k <= ny
        cover[s, r0:r0 + k] += 1
    assert (cover == 1).all()


def test_equal_costs_give_equal_groups(L):
    m16 = mask_words(basins()['box'])
    t = plan(L, 2, m16, 16, 1.0)
    for s in np.unique(t[t[:, 2] > 0, 0]):
        k = t[(t[:, 0] == s) & (t[:, 2] > 0), 2]
        assert (k[:-1] == 16).all() and 1 <= k[-1] <= 16


def test_coastal_strips_get_shorter_groups_as_their_cost_rises(L):
    box = np.ones((300, 200), bool)
    box[:, 0] = box[:, -1] = False  # west and east coasts, open north and south
    m16 = mask_words(box)
    groups = {}
    for cost in (1.0, 1.5, 2.5):
        t = plan(L, 2, m16, 16, cost)
        t = t[t[:, 2] > 0]
        groups[cost] = [int((t[:, 0] == s).sum()) for s in range(strips_of(2, 200))]
    interior = strips_of(2, 200) // 2
    assert groups[1.0][0] == groups[1.0][interior]
    assert groups[1.0][0] < groups[1.5][0] < groups[2.5][0]
    assert groups[1.0][interior] == groups[2.5][interior]


@pytest.mark.parametrize('ny', [1, 2, 3, 4])
def test_basins_of_a_few_rows(L, ny):
    m16 = mask_words(np.ones((ny, 40), bool))
    for rows, cost in ((4, 1.0), (16, 2.6)):
        t = plan(L, 2, m16, rows, cost)
        t = t[t[:, 2] > 0]
        cover = np.zeros((strips_of(2, 40), ny), int)
        for s, r0, k in t:
            cover[s, r0:r0 + k] += 1
        assert (cover == 1).all()


def test_bad_arguments_are_refused(L):
    m16 = mask_words(basins()['ocean'])
    p = m16.ctypes.data_as(ctypes.c_void_p)
    assert L.swm_gpu_plan_step_tiles(2, 0, 40, p, 16, 1.0, None, 0) == -1
    assert L.swm_gpu_plan_step_tiles(2, 61, 40, None, 16, 1.0, None, 0) == -1
    assert L.swm_gpu_plan_step_tiles(2, 61, 40, p, 0.5, 1.0, None, 0) == -1
    assert L.swm_gpu_plan_step_tiles(2, 61, 40, p, 16, 0.5, None, 0) == -1
    assert L.swm_gpu_plan_step_tiles(2, 61, 40, p, 16, 1.0, None, 4) == -1
    assert L.swm_gpu_plan_step_tiles(2, 1, 1 << 23, p, 16, 1.0, None, 0) == -1
