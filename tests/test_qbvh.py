"""CPU: the quantized 4-wide BLAS layout (wf_init_params.blas_layout = 1).

wf_bvh_quantize (host code of the library, no GPU needed) collapses a binary
BLAS blob into 64-byte nodes of up to four children with 8-bit planes.  The
traversal's parity with the exact binary tree rests on two properties checked
here on the blobs of the configurations' meshes: every dequantized child box
(computed in float exactly as the kernel computes it) contains the child's
exact box, and the collapse references every binary leaf once, with its
triangle range unchanged.  And the oracle's tie rule that the layout's
closest hits follow changes no hit on these scenes (no exact-t ties).
"""
import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300 import scenes
from tests.helpers import oracle_scene_from_desc


def binary_nodes(blob):
    h = blob[:12].view(np.uint32)
    n = (h[1] - 12) // 32
    raw = blob[12:12 + 32 * n]
    f = raw.view(np.float32).reshape(n, 8)
    u = raw.view(np.uint32).reshape(n, 8)
    return f[:, 0:3], f[:, 4:7], u[:, 3], u[:, 7]   # min, max, left_first, prim_count


def decode(words, k):
    w = words[16 * k:16 * k + 16]
    origin = w[0:3].view(np.float32)
    meta = int(w[3])
    scale = [np.uint32(((meta >> (8 * a)) & 0xFF) << 23).view(np.float32) for a in range(3)]
    nch = meta >> 24
    kids = []
    for i in range(nch):
        lo = np.array([origin[a] + np.float32((int(w[4 + a]) >> (8 * i)) & 0xFF) * scale[a] for a in range(3)],
                      np.float32)
        hi = np.array([origin[a] + np.float32((int(w[8 + a]) >> (8 * i)) & 0xFF) * scale[a] for a in range(3)],
                      np.float32)
        count = ((int(w[7]) >> (8 * i)) & 0xFF) | (((int(w[11]) >> (8 * i)) & 0xFF) << 8)
        kids.append((lo, hi, int(w[12 + i]), count))
    return kids


def decode_exact(words, k):
    w = words[32 * k:32 * k + 32]
    planes = w[0:24].view(np.float32).reshape(3, 2, 4)   # axis, lo / hi, child
    nch = int(w[28]) >> 24
    kids = []
    for i in range(nch):
        lo = np.array([planes[a, 0, i] for a in range(3)], np.float32)
        hi = np.array([planes[a, 1, i] for a in range(3)], np.float32)
        count = int(w[28 + i]) & (0x00FFFFFF if i == 0 else 0xFFFFFFFF)
        kids.append((lo, hi, int(w[24 + i]), count))
    return kids


def check_blob(blob, exact=False):
    words, root_count = (wf.bvh_widen if exact else wf.bvh_quantize)(blob)
    stride = 32 if exact else 16
    mn, mx, lf, pc = binary_nodes(blob)
    if pc[0] > 0:
        assert root_count == pc[0] and len(words) == 0
        return 0
    assert root_count == 0
    seen_leaves = []
    order = [0]   # qnode indices follow the collapse in pre-order

    def walk(bi, qk):
        kids_b = []
        for c in (lf[bi], lf[bi] + 1):
            if pc[c] > 0:
                kids_b.append(c)
            else:
                kids_b += [lf[c], lf[c] + 1]
        kids_q = (decode_exact if exact else decode)(words, qk)
        assert len(kids_q) == len(kids_b)
        for (lo, hi, child, count), b in zip(kids_q, kids_b):
            if exact:   # the binary boxes, bit for bit
                assert np.array_equal(lo.view(np.uint32), mn[b].view(np.uint32))
                assert np.array_equal(hi.view(np.uint32), mx[b].view(np.uint32))
            else:       # quantized outward
                assert np.all(lo <= mn[b]) and np.all(hi >= mx[b]), (lo, mn[b], hi, mx[b])
            assert count == pc[b]
            if pc[b] > 0:
                assert child == lf[b]
                seen_leaves.append(b)
            else:
                order.append(order[-1] + 1)
                assert child == order[-1]
                walk(b, child)

    walk(0, 0)
    assert len(words) == stride * len(order)
    leaves = np.nonzero(pc > 0)[0]
    # node 1 is the reference's unused slot; every other leaf once
    assert sorted(seen_leaves) == sorted(x for x in leaves if x != 1)
    return len(order)


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("name", ["box", "instanced", "soup"])
def test_quantized_boxes_contain_the_exact_boxes(orc, name, exact):
    """Both 4-wide layouts reference every binary leaf once with its triangle
    range; the quantized boxes contain the exact ones, the exact layout's
    boxes are the binary ones bit for bit."""
    if name == "box":
        meshes = scenes.box_scene(width=8, height=8).meshes
    elif name == "instanced":
        meshes = scenes.instanced_scene(width=8, height=8, instances=8, freqs=(20, 33), spp=1).meshes
    else:
        meshes = [scenes.triangle_soup(50_000, seed=7)]
    for t in meshes:
        for bins, leaf in ((16, 4), (8, 0)):
            blob = orc.bvh_build(t, bins, False, leaf)
            n = check_blob(blob, exact)
            if len(t) > 8:
                assert n > 0


def test_single_leaf_blas_has_no_nodes(orc):
    t = scenes.quad((0, 0, 0), (1, 0, 0), (0, 1, 0))
    blob = orc.bvh_build(t, 8, False, 0)
    for fn in (wf.bvh_quantize, wf.bvh_widen):
        words, root_count = fn(blob)
        assert len(words) == 0 and root_count == 2


def test_rejects_a_truncated_blob(orc):
    blob = orc.bvh_build(scenes.icosphere(4), 16, False, 4)
    with pytest.raises(wf.WFError):
        wf.bvh_quantize(blob[:20])
    with pytest.raises(wf.WFError):
        wf.bvh_widen(blob[:20])


def test_tie_rule_changes_no_hit_on_the_configurations(orc):
    """The tie rule (smallest t, then smallest instance / primitive) picks the
    same hits as the reference's first-found order wherever no two triangles
    give exactly the same t."""
    from tests.test_ref_hlsl import random_rays
    for desc, lo, hi in ((scenes.box_scene(width=96, height=96), 0.02, 0.98),
                         (scenes.instanced_scene(width=96, height=54, instances=64, freqs=(6, 9, 12, 15), spp=1),
                          0.0, 100.0)):
        sc = oracle_scene_from_desc(orc, desc)
        rays = np.concatenate([orc.primary_rays(desc.view, desc.width, desc.height), random_rays(20000, lo, hi, 3)])
        a, _, _ = sc.trace(rays, threads=8)
        b, _, _ = sc.trace(rays, flags=orc.TIE_RULE, threads=8)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
