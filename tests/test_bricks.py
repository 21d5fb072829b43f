"""Host side of the brick tiling (no GPU): the ranked brick shapes of the
cost model and ragged bricks for grids the brick side does not divide."""
import math

import numpy as np

import lcpgrid as L


def _ucell(ngrid, side=11.0, rc=7.0, natom=3, no=13):
    pos = np.array([[1.0, 2.0, 3.0], [5.5, 6.0, 8.5], [8.0, 1.5, 6.0]])[:natom]
    return L.UCell(1, np.eye(3) * side, natom, [1] * natom, pos, [rc] * natom, ngrid, [0, 0, 0],
                   Total_NumOrbs=[no] * natom)


def test_candidates_ranked_and_within_limits():
    u = _ucell((44, 40, 48))
    cands = u.brick_shape_candidates(64)
    assert len(cands) > 10
    costs = [c for _, c in cands]
    assert costs == sorted(costs)
    for shape, _ in cands:
        assert all(1 <= b <= 8 for b in shape)
        assert 16 <= math.prod(shape) <= 128
    # the best shapes fill most of the 128 point slots of an MMA tile
    assert math.prod(cands[0][0]) >= 96


def test_candidates_respect_small_grids():
    u = _ucell((5, 6, 7), side=4.0, rc=3.0, natom=1, no=4)
    for shape, _ in u.brick_shape_candidates(100):
        assert shape[0] <= 5 and shape[1] <= 6 and shape[2] <= 7


def test_ragged_bricks_cover_the_grid():
    u = _ucell((45, 42, 49))
    info = u.brick_info()
    bd, nb = info["bdim"], info["nbricks_axis"]
    assert tuple(bd) == u.brick_shape_candidates(1)[0][0]
    for d in range(3):
        assert nb[d] == -(-u.Ngrid[d] // bd[d])  # ceil: the last brick of an axis may be ragged
    assert info["bricks"] == nb[0] * nb[1] * nb[2]
    assert info["points"] == bd[0] * bd[1] * bd[2]
    assert 0 < info["max_images"] <= 512
