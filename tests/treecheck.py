"""Structural checks of a BVHNode array (test helper)."""
import numpy as np

LEAF = np.int64(0x80000000)


def check_tree(nodes, n_prims, boxes_of_prims=None):
    """Raise AssertionError unless `nodes` is a binary BVH over n_prims leaves with the root at 0:
    2n-1 nodes, every node reached once, every primitive in exactly one leaf, leaf right = -1,
    every child box inside its parent box."""
    nn = nodes.shape[0]
    if n_prims == 0:
        assert nn == 0
        return
    assert nn == 2 * n_prims - 1, (nn, n_prims)
    left = nodes["left"].astype(np.int64)
    right = nodes["right"].astype(np.int64)
    leaf = left < 0
    assert leaf.sum() == n_prims
    assert np.all(right[leaf] == -1)
    prims = (left[leaf] & 0x7FFFFFFF)
    assert np.array_equal(np.sort(prims), np.arange(n_prims))
    internal = ~leaf
    ch = np.concatenate([left[internal], right[internal]])
    assert np.all((ch >= 0) & (ch < nn))
    cnt = np.bincount(ch, minlength=nn)
    assert cnt[0] == 0, "root must not be a child"
    assert np.all(cnt[1:] == 1), "every non-root node has exactly one parent"
    mn, mx = nodes["min"], nodes["max"]
    for c in (left, right):
        p = np.nonzero(internal)[0]
        cc = c[internal]
        assert np.all(mn[cc] >= mn[p]) and np.all(mx[cc] <= mx[p]), "child box outside parent"
    if boxes_of_prims is not None:
        pl = prims
        assert np.array_equal(mn[leaf].view(np.uint32), boxes_of_prims["min"][pl].view(np.uint32))
        assert np.array_equal(mx[leaf].view(np.uint32), boxes_of_prims["max"][pl].view(np.uint32))
