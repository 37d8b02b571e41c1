"""The rule behind the single-image chain's one-labelling hole fill, checked on the CPU.

With dual connectivities (foreground 8-connected and background 4-connected, or the other way
round) the components of a binary image and of its complement form a tree by enclosure, and a
component's parent is the component of the pixel directly above its first pixel in raster
order.  The device labels both classes in one forest and joins every component to its parent
unless the parent is a background component touching the border; the sets that result must be
the components of the filled image (foreground plus its holes), labelled in raster order.

This test restates that rule with scipy on random images and compares it with the direct
statement (fill the holes, then label the filled image), for both dual pairs.  With 4 and 4 the
rule fails on many images, which shows the test can tell a wrong rule apart; the device takes
the rule only for the dual pairs and labels twice otherwise.
"""
import numpy as np
import pytest

ndi = pytest.importorskip("scipy.ndimage")

S4 = ndi.generate_binary_structure(2, 1)
S8 = ndi.generate_binary_structure(2, 2)


def _struct(conn):
    return S8 if conn == 8 else S4


def fill_then_label(fg, fill_conn, label_conn):
    """imfillHoles(fg, fill_conn) then bwlabel(label_conn), raster-numbered."""
    bg_lab, _ = ndi.label(~fg, _struct(fill_conn))
    edge = np.concatenate([bg_lab[0], bg_lab[-1], bg_lab[:, 0], bg_lab[:, -1]])
    outside = np.isin(bg_lab, np.unique(edge[edge > 0]))
    filled = fg | ~outside
    labels, n = ndi.label(filled, _struct(label_conn))  # scipy numbers in raster order
    return filled, labels, n


def tree_rule(fg, fill_conn, label_conn):
    """One forest over both classes, each component joined to the component above its first
    pixel unless that one (or the component itself) is a background component on the border."""
    H, W = fg.shape
    fl, nf = ndi.label(fg, _struct(label_conn))
    bl, nb = ndi.label(~fg, _struct(fill_conn))
    comp = np.where(fg, fl, bl + nf).ravel()  # 1..nf foreground, nf+1.. background
    first = np.full(nf + nb + 1, -1)
    ids, idx = np.unique(comp, return_index=True)
    first[ids] = idx
    grid = comp.reshape(H, W)
    edge = np.concatenate([grid[0], grid[-1], grid[:, 0], grid[:, -1]])
    outside = set(int(c) for c in np.unique(edge) if c > nf)
    parent = np.arange(nf + nb + 1)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for c in range(1, nf + nb + 1):
        if c in outside:
            continue
        y, x = divmod(int(first[c]), W)
        if y == 0:
            continue  # a foreground component on the first row: its parent is the outside
        p = int(grid[y - 1, x])
        if p in outside:
            continue
        a, b = find(c), find(p)
        if a != b:
            # keep the root with the smaller first pixel, as the device's atomicMin hooking does
            if first[a] < first[b]:
                a, b = b, a
            parent[a] = b
    root = np.array([find(c) for c in range(nf + nb + 1)])
    r = root[comp]
    is_out = np.isin(comp, list(outside)) if outside else np.zeros(comp.shape, bool)
    filled = ~is_out.reshape(H, W)
    # raster relabel of the roots of filled pixels
    roots_in_order = []
    seen = set()
    for i in np.flatnonzero(~is_out):
        if r[i] not in seen:
            seen.add(r[i])
            roots_in_order.append(r[i])
    rank = {v: k + 1 for k, v in enumerate(roots_in_order)}
    labels = np.array([rank.get(v, 0) if not o else 0 for v, o in zip(r, is_out)], np.int64).reshape(H, W)
    return filled, labels, len(roots_in_order)


def _images(rng, count):
    for _ in range(count):
        h, w = rng.integers(1, 20, 2)
        yield rng.random((h, w)) < rng.uniform(0.25, 0.75)


@pytest.mark.parametrize("fill_conn,label_conn", [(4, 8), (8, 4)])
def test_tree_rule_matches_fill_then_label(fill_conn, label_conn):
    rng = np.random.default_rng(1234)
    for fg in _images(rng, 600):
        f0, l0, n0 = fill_then_label(fg, fill_conn, label_conn)
        f1, l1, n1 = tree_rule(fg, fill_conn, label_conn)
        assert np.array_equal(f0, f1) and np.array_equal(l0, l1) and n0 == n1, fg.astype(int)


def test_tree_rule_fails_for_four_and_four():
    rng = np.random.default_rng(99)
    mismatches = 0
    for fg in _images(rng, 300):
        f0, l0, n0 = fill_then_label(fg, 4, 4)
        f1, l1, n1 = tree_rule(fg, 4, 4)
        mismatches += not (np.array_equal(f0, f1) and np.array_equal(l0, l1) and n0 == n1)
    assert mismatches > 0
