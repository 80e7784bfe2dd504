"""The reference's spatial partitioners restated in float32 Python, as the
checker of the partitioned join's partitioning: the KDB tree
(rust/sedona-spatial-join/src/partitioning/kdb.rs: insert_rect, split,
assign_leaf_ids, partition_no_multi), rect_intersection_area and
rects_intersect (partitioning/util.rs), and the flat partitioner over
partition bounds (partitioning/flat.rs: partition)."""
import numpy as np

F = np.float32


class _Node:
    def __init__(self, ext, level):
        self.ext = [F(v) for v in ext]
        self.level = level
        self.items = []
        self.children = None
        self.leaf = -1


def _contains(ext, x, y):
    return ext[0] <= x <= ext[2] and ext[1] <= y <= ext[3]


class Kdb:
    def __init__(self, max_items, max_levels, extent):
        self.max_items, self.max_levels = max_items, max_levels
        self.root = _Node(extent, 0)

    def insert(self, r):
        r = [F(v) for v in r]
        if _contains(self.root.ext, r[0], r[1]):
            self._insert(self.root, r)

    def _insert(self, node, r):
        if node.children is None:
            if len(node.items) < self.max_items or node.level >= self.max_levels:
                node.items.append(r)
                return
            e = node.ext
            sx = (e[2] - e[0]) > (e[3] - e[1])
            if not self._split(node, sx) and not self._split(node, not sx):
                node.items.append(r)
                return
        for c in node.children:
            if _contains(c.ext, r[0], r[1]):
                self._insert(c, r)
                break

    def _split(self, node, sx):
        key = (lambda r: (r[0], r[1])) if sx else (lambda r: (r[1], r[0]))
        node.items.sort(key=key)  # stable, as Rust's sort_by
        mid = node.items[len(node.items) // 2]
        c = mid[0] if sx else mid[1]
        e = node.ext
        if sx and (c <= e[0] or c >= e[2]):
            return False
        if not sx and (c <= e[1] or c >= e[3]):
            return False
        if sx:
            left, right = [e[0], e[1], c, e[3]], [c, e[1], e[2], e[3]]
        else:
            left, right = [e[0], e[1], e[2], c], [e[0], c, e[2], e[3]]
        lc, rc = _Node(left, node.level + 1), _Node(right, node.level + 1)
        items, node.items = node.items, []
        for it in items:
            self._insert(lc if (it[0] if sx else it[1]) <= c else rc, it)
        node.children = [lc, rc]
        return True

    def leaves(self):
        out = []

        def walk(n):
            if n.children is None:
                n.leaf = len(out)
                out.append(n.ext)
            else:
                for c in n.children:
                    walk(c)

        walk(self.root)
        return np.array(out, dtype=F).reshape(-1, 4)


def no_multi(boxes, leaves):
    """partition_no_multi: the leaf each box overlaps most, first in leaf
    order on a tie; 0xFFFFFFFF for NaN boxes and boxes meeting no leaf."""
    b = boxes.astype(F)[:, None, :]
    L = leaves.astype(F)[None, :, :]
    meet = (L[..., 0] <= b[..., 2]) & (L[..., 2] >= b[..., 0]) & \
           (L[..., 1] <= b[..., 3]) & (L[..., 3] >= b[..., 1])
    w = np.maximum(np.minimum(b[..., 2], L[..., 2]) - np.maximum(b[..., 0], L[..., 0]), F(0))
    h = np.maximum(np.minimum(b[..., 3], L[..., 3]) - np.maximum(b[..., 1], L[..., 1]), F(0))
    area = np.where(meet, (w * h).astype(F), F(-1))
    best = np.argmax(area, axis=1).astype(np.uint32)
    best[~meet.any(axis=1)] = 0xFFFFFFFF
    return best


def flat(boxes, bounds):
    """FlatPartitioner::partition: the one bound met, len(bounds) (Multi) for
    several, len(bounds) + 1 (None) for none."""
    b = boxes.astype(F)[:, None, :]
    B = bounds.astype(F)[None, :, :]
    meet = (B[..., 0] <= b[..., 2]) & (B[..., 2] >= b[..., 0]) & \
           (B[..., 1] <= b[..., 3]) & (B[..., 3] >= b[..., 1])
    cnt = meet.sum(axis=1)
    out = np.argmax(meet, axis=1).astype(np.uint32)
    out[cnt > 1] = len(bounds)
    out[cnt == 0] = len(bounds) + 1
    return out
