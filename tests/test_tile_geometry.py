"""Index arithmetic of the materialisation's shared-memory tiles (CPU).

A restatement of `materialize_kernel`'s staging (webgpu_bfs_gb300/csrc/
level_kernels.cu, MatGeo): each of the 256 threads moves four consecutive
tile words of every array into shared memory at [word][vertex], and each of
the 16 (word, 64-vertex segment) columns is read back as 8-byte pairs. The
test checks, for every compiled word width and ragged vertex counts, that
every global access is in bounds and 16-byte aligned when vectorised
(including the plane bases, b*V*W words into their buffer), that every
shared index stays inside its array, that no two threads write one slot,
and that each column read sees exactly the (vertex, word) it stands for.
"""
import pytest

MAT_BLOCK = 256
TILE = MAT_BLOCK * 4


def _geo(W):
    tw = W if W <= 16 else 16
    tv = TILE // tw
    rs = tv + 2
    return tw, tv, rs, tw * rs


@pytest.mark.parametrize("W", [1, 2, 4, 8, 16, 32, 64])
def test_tile_staging_indices(W):
    tw, tv, rs, arr = _geo(W)
    assert tw * (tv // 64) == 16 and rs % 2 == 0 and arr % 2 == 0
    for V in (1, 3, 5, 63, 65, 1001, 1025, 2050):
        VW = V * W
        vec_planes = VW % 4 == 0
        for P in sorted({1, 33, 32 * W - 1, 32 * W}):
            if P > 32 * W:
                continue
            Wu = (P + 31) // 32
            ngu = (Wu + tw - 1) // tw
            for it in range(((V + tv - 1) // tv) * ngu):
                g, v0 = it % ngu, (it // ngu) * tv
                sh = {}
                for tid in range(MAT_BLOCK):
                    o = 4 * tid
                    if W <= 16:
                        gw, inb = v0 * W + o, v0 * W + o + 3 < VW
                    else:
                        gw, inb = (v0 + o // 16) * W + 16 * g + o % 16, v0 + o // 16 < V
                    for plane in range(8):
                        if inb and vec_planes:
                            assert (plane * VW + gw) % 4 == 0
                    assert gw % 4 == 0
                    for k in range(4):
                        idx = ((o + k) % tw) * rs + (o + k) // tw
                        assert 0 <= idx < arr and idx not in sh
                        if inb or (W <= 16 and gw + k < VW):
                            assert gw + k < VW
                            if W <= 16:
                                sh[idx] = ((gw + k) // W, (gw + k) % W)
                            else:
                                sh[idx] = (v0 + o // 16, 16 * g + o % 16 + k)
                        else:
                            sh[idx] = None
                for cs in range(16):
                    c, seg = cs % tw, cs // tw
                    if g * tw + c >= Wu:
                        continue
                    for lane in range(32):
                        vloc = seg * 64 + 2 * lane
                        assert vloc + 1 < tv
                        for t in range(2):
                            got = sh.get(c * rs + vloc + t)
                            if v0 + vloc + t < V:
                                assert got == (v0 + vloc + t, g * tw + c)
                            else:
                                assert got is None
