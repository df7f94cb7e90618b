"""Index arithmetic of the cluster-mode CTA kernel (CPU).

A restatement of `cta_cluster_kernel` and `cta_cluster_shape`
(webgpu_bfs_gb300/csrc/cta_kernel.cu): rank r of a CL-block cluster keeps
bitmap words [r*wpb, (r+1)*wpb), wpb = ceil(words / CL); a word w belongs
to rank w / wpb at offset w - rank*wpb; each rank fills the unreached
vertices [32*w0, min(V, 32*w1)) of its slice; the queue halves follow the
slice in shared memory. For the vertex counts that pick cluster mode, the
test checks that the owner rank exists, the offsets stay inside a slice,
the slices partition the bitmap and the fills partition the vertices, and
that slice plus queue halves fit one block's shared memory.
"""
import pytest

OPTIN = 232448          # max dynamic shared memory per block (227 KB)
SLACK = 2048
CTA_SMEM_QUEUE = 4096


def shape(V, entry):
    """The cluster size and shared memory cta_cluster_shape picks (None:
    the bitmap does not fit 8 slices)."""
    words = (V + 31) // 32
    for cl in (2, 4, 8):
        wpb = (words + cl - 1) // cl
        slice_ = (wpb + 1) // 2 * 2 * 4
        if slice_ + 2 * 1024 * entry + SLACK > OPTIN:
            continue
        room = OPTIN - SLACK - slice_
        qh = min(CTA_SMEM_QUEUE, room // (2 * entry) // 32 * 32)
        return cl, wpb, slice_, qh, slice_ + 2 * qh * entry
    return None


@pytest.mark.parametrize("V", [1_851_393, 1_960_000, 2_096_704, 2_250_000, 4_000_000,
                               7_000_001, 9_000_000, 13_697_024])
@pytest.mark.parametrize("entry", [4, 8])  # vertex ids / edge-record ranges
def test_cluster_slices_and_fills(V, entry):
    got = shape(V, entry)
    assert got is not None, "cluster mode must cover this V"
    cl, wpb, slice_, qh, smem = got
    words = (V + 31) // 32
    assert smem <= OPTIN - SLACK and qh >= 1024 and qh % 32 == 0
    assert slice_ % 8 == 0  # queue halves start 8-byte aligned (edge ranges)
    # slices: [w0, w1) per rank, as the kernel computes them
    bounds = [(min(words, r * wpb), min(words, min(words, r * wpb) + wpb)) for r in range(cl)]
    assert bounds[0][0] == 0 and bounds[-1][1] == words
    for (a0, a1), (b0, b1) in zip(bounds, bounds[1:]):
        assert a1 == b0
    for w in (0, 1, wpb - 1, wpb, words // 2, words - 1):
        o = w // wpb
        assert 0 <= o < cl
        assert 0 <= w - o * wpb < wpb and (w - o * wpb) * 4 < slice_
    # fills: [32*w0, min(V, 32*w1)) per rank partition [0, V)
    fills = [(32 * w0, min(V, 32 * w1)) for w0, w1 in bounds]
    assert fills[0][0] == 0 and fills[-1][1] == V
    for (a0, a1), (b0, b1) in zip(fills, fills[1:]):
        assert a1 == b0


def test_cluster_capacity_limit():
    # 8 slices of at most OPTIN - SLACK - 2*1024*entry bytes bound the vertex
    # count: 13,697,024 with edge-range entries, 14,221,312 with vertex ids
    assert shape(13_697_024, 8) is not None and shape(13_697_025, 8) is None
    assert shape(14_221_312, 4) is not None and shape(14_221_313, 4) is None
