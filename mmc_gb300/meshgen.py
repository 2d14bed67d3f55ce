"""Tetrahedral mesh recipes for the photon-tracing workloads.

Every workload mesh is a structured cube split into 6 tetrahedra per voxel (the
Kuhn split used by the reference's built-in ``dmmc-cube60`` benchmark,
``src/mmc_bench.c:61-78``: corner order (0,0,0),(1,0,0),(0,1,0),(1,1,0),(0,0,1),
(1,0,1),(0,1,1),(1,1,1) and tets [1,2,8,4],[1,3,4,8],[1,2,6,8],[1,5,8,6],
[1,3,8,7],[1,5,7,8]).  Interior nodes may be jittered to make the tets
irregular; the jitter is orientation-safe: a node is re-drawn until every tet
touching it keeps at least ``min_ratio`` of its undeformed volume (uniform
+/-0.25 mm jitter on a 1 mm grid otherwise inverts a few tets, and the
reference's tracer never terminates on an inverted tet).

Arrays follow the reference's mesh conventions (``src/mmc_mesh.h:87-122``):
``node`` float32 (nn, 3); ``elem`` int32 (ne, 4), 1-based; ``label`` int32 (ne,),
0 = void/background; media rows are (mua, mus, g, n) with row 0 the background.
"""
from __future__ import annotations

import dataclasses
import numpy as np

# local corner coordinates of a voxel, 0-based corner ids 0..7
_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0],
                     [0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]], dtype=np.int64)
_KUHN6 = np.array([[1, 2, 8, 4], [1, 3, 4, 8], [1, 2, 6, 8],
                   [1, 5, 8, 6], [1, 3, 8, 7], [1, 5, 7, 8]], dtype=np.int64) - 1


@dataclasses.dataclass
class Mesh:
    node: np.ndarray          # (nn,3) float32
    elem: np.ndarray          # (ne,4) int32, 1-based
    label: np.ndarray         # (ne,) int32
    media: np.ndarray         # (nmedia+1, 4) float32 rows (mua, mus, g, n)
    name: str = "mesh"

    @property
    def nn(self) -> int:
        return int(self.node.shape[0])

    @property
    def ne(self) -> int:
        return int(self.elem.shape[0])


def kuhn_cube(n: int, h: float, origin=(0.0, 0.0, 0.0)):
    """Structured cube of n^3 voxels of edge h, 6 tets per voxel.

    Node ids run x fastest, then y, then z; tets run voxel by voxel (x fastest)
    with the six Kuhn tets of a voxel consecutive.
    """
    m = n + 1
    ii = np.arange(m, dtype=np.float64)
    zz, yy, xx = np.meshgrid(ii, ii, ii, indexing="ij")
    node = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1) * h
    node += np.asarray(origin, dtype=np.float64)[None, :]
    vv = np.arange(n, dtype=np.int64)
    vz, vy, vx = np.meshgrid(vv, vv, vv, indexing="ij")
    base = (vx + m * vy + m * m * vz).ravel()
    off = _CORNERS[:, 0] + m * _CORNERS[:, 1] + m * m * _CORNERS[:, 2]
    elem = base[:, None, None] + off[_KUHN6][None, :, :]
    elem = elem.reshape(-1, 4) + 1
    return node, elem.astype(np.int32)


def signed_volumes(node: np.ndarray, elem: np.ndarray) -> np.ndarray:
    """Signed volume (1/6 of the triple product) of each tet, float64."""
    p = node.astype(np.float64)
    e = elem.astype(np.int64) - 1
    a, b, c, d = p[e[:, 0]], p[e[:, 1]], p[e[:, 2]], p[e[:, 3]]
    return np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) / 6.0


def jitter_nodes(node, elem, n, amp, seed, min_ratio=0.1, max_iter=200):
    """Uniform +/-amp jitter of interior nodes, re-drawn where a tet would shrink
    below ``min_ratio`` of its undeformed (signed) volume."""
    rng = np.random.default_rng(seed)
    m = n + 1
    idx = np.arange(m ** 3)
    ix, iy, iz = idx % m, (idx // m) % m, idx // (m * m)
    interior = (ix > 0) & (ix < n) & (iy > 0) & (iy < n) & (iz > 0) & (iz < n)
    base = node.astype(np.float64)
    vol0 = signed_volumes(base, elem)
    out = base.copy()
    todo = np.nonzero(interior)[0]
    for _ in range(max_iter):
        out[todo] = base[todo] + rng.uniform(-amp, amp, size=(todo.size, 3))
        ratio = signed_volumes(out, elem) / vol0
        bad = np.nonzero(ratio <= min_ratio)[0]
        if bad.size == 0:
            return out
        cand = np.unique(elem[bad].ravel() - 1)
        todo = cand[interior[cand]]
    raise RuntimeError("jitter could not keep all tets positively oriented")


def centroids(node, elem):
    return node.astype(np.float64)[elem.astype(np.int64) - 1].mean(axis=1)


# ---------------------------------------------------------------------------
# workload recipes
# ---------------------------------------------------------------------------

C0_MEDIA = np.array([[0.0, 0.0, 1.0, 1.0],
                     [0.005, 1.0, 0.01, 1.37]], dtype=np.float32)
C1_MEDIA = np.array([[0.0, 0.0, 1.0, 1.0],
                     [0.005, 1.0, 0.01, 1.37],
                     [0.05, 5.0, 0.9, 1.37]], dtype=np.float32)
SHELL_MEDIA = np.array([[0.0, 0.0, 1.0, 1.0],
                        [0.02, 1.0, 0.9, 1.37],
                        [0.004, 0.01, 0.9, 1.37],
                        [0.016, 8.6, 0.9, 1.37],
                        [0.019, 7.8, 0.89, 1.37]], dtype=np.float32)
SHELL_RADII = (18.0, 20.0, 23.0, 25.0)


def homogeneous_cube(n=30, size=60.0, media=C0_MEDIA, name="cube"):
    """Homogeneous cube [0,size]^3 with n^3 voxels (162,000 tets at n=30)."""
    node, elem = kuhn_cube(n, size / n)
    label = np.ones(elem.shape[0], dtype=np.int32)
    return Mesh(node.astype(np.float32), elem, label, np.array(media, np.float32), name)


def inclusion_cube(n=60, size=60.0, jitter=0.25, seed=12345, radius=10.0,
                   center=(30.0, 30.0, 30.0), media=C1_MEDIA, name="inclusion"):
    """Jittered cube with a spherical inclusion labelled 2 (1,296,000 tets at n=60)."""
    node, elem = kuhn_cube(n, size / n)
    if jitter > 0:
        node = jitter_nodes(node, elem, n, jitter, seed)
    c = centroids(node, elem)
    r = np.linalg.norm(c - np.asarray(center)[None, :], axis=1)
    label = np.where(r < radius, 2, 1).astype(np.int32)
    return Mesh(node.astype(np.float32), elem, label, np.array(media, np.float32), name)


def shell_mesh(n=60, size=60.0, jitter=0.25, seed=4321, media=SHELL_MEDIA,
               radii=SHELL_RADII, center=(30.0, 30.0, 30.0), name="shells"):
    """Four concentric spherical shells; tets beyond the outer radius are void (0)."""
    node, elem = kuhn_cube(n, size / n)
    if jitter > 0:
        node = jitter_nodes(node, elem, n, jitter, seed)
    c = centroids(node, elem)
    r = np.linalg.norm(c - np.asarray(center)[None, :], axis=1)
    label = np.zeros(elem.shape[0], dtype=np.int32)
    for k in range(len(radii) - 1, -1, -1):
        label[r < radii[k]] = k + 1
    return Mesh(node.astype(np.float32), elem, label, np.array(media, np.float32), name)


def c1_detectors():
    """4 detectors of radius 2 mm on z=0, 10/15/20/25 mm from the (30,30,0) source."""
    return np.array([[40.0, 30.0, 0.0, 2.0], [45.0, 30.0, 0.0, 2.0],
                     [50.0, 30.0, 0.0, 2.0], [55.0, 30.0, 0.0, 2.0]], dtype=np.float32)
