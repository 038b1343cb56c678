"""The per-mother BVH of the flattened scene (surface-area-heuristic splits):
every daughter sits in exactly one leaf, every box holds what lies below it,
the depth leaves room in the device's 32-entry traversal stack, and on the
Davies-Cotton dish a vertical ray overlaps only a handful of the 380 facet
boxes (a median split on the camera-stretched z axis had cut the dish into
rings spanning all of it)."""
import numpy as np
import pytest

from robast_gb300 import configs


def _walk(fl, root):
    """(leaf items, max depth, [(node box, child boxes or item ids)])"""
    items, depth, pairs = [], 0, []
    stack = [(root, 0)]
    while stack:
        i, d = stack.pop()
        depth = max(depth, d)
        b = fl.bvh[i]
        lo, hi = np.array(b.lo[:]), np.array(b.hi[:])
        if b.left < 0:
            ids = [fl.bvh_items[b.item_begin + k] for k in range(b.right)]
            items += ids
            pairs.append((lo, hi, "items", ids))
        else:
            pairs.append((lo, hi, "nodes", [b.left, b.right]))
            stack += [(b.left, d + 1), (b.right, d + 1)]
    return items, depth, pairs


@pytest.mark.parametrize("name,kw", [("davies_cotton", dict(n_rays=10)), ("light_guide", dict(n_rays=10)),
                                     ("schmidt_cassegrain", dict(n_rays=10, n_samples=64))])
def test_bvh_structure(name, kw):
    man, _ = configs.CONFIGS[name](**kw)
    fl = man._ensure_scene().flat
    checked = 0
    for m in range(fl.n_nodes):
        nd = fl.nodes[m]
        if nd.bvh_root < 0:
            continue
        checked += 1
        children = sorted(fl.children[nd.child_begin + k] for k in range(nd.child_count))
        items, depth, pairs = _walk(fl, nd.bvh_root)
        assert sorted(items) == children  # each daughter exactly once
        assert depth < 28  # the traversal stack holds depth + 1 entries
        for lo, hi, kind, ids in pairs:
            if kind == "items":
                assert len(ids) <= 4
                for c in ids:
                    assert (np.array(fl.nodes[c].lo[:]) >= lo).all() and (np.array(fl.nodes[c].hi[:]) <= hi).all()
            else:
                for j in ids:
                    b = fl.bvh[j]
                    assert (np.array(b.lo[:]) >= lo).all() and (np.array(b.hi[:]) <= hi).all()
    assert checked >= 1


def test_vertical_rays_overlap_few_facets():
    man, _ = configs.davies_cotton(n_rays=10, n_facets=380)
    fl = man._ensure_scene().flat
    root = fl.nodes[0].bvh_root
    g = np.random.default_rng(0)
    tested = []
    for x, y in g.uniform(-600, 600, (500, 2)):
        n_items, stack = 0, [root]
        while stack:
            b = fl.bvh[stack.pop()]
            if not (b.lo[0] <= x <= b.hi[0] and b.lo[1] <= y <= b.hi[1]):
                continue
            if b.left < 0:
                n_items += b.right
            else:
                stack += [b.left, b.right]
        tested.append(n_items)
    assert np.mean(tested) < 8, np.mean(tested)
