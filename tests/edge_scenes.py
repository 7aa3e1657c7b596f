"""Hand-built scenes and rays that exercise the corners of the ray-query contract."""
import numpy as np

from selas_gb300 import make_rayhits, make_rays
from selas_gb300.scenes import TriangleScene


def grid_scene(n=8):
    """A unit-spaced n x n quad grid in the plane y = 0 (2 triangles per quad, shared edges and vertices),
    a duplicate of one quad under another geomID, and a zero-area triangle."""
    xs, zs = np.meshgrid(np.arange(n + 1, dtype=np.float32), np.arange(n + 1, dtype=np.float32), indexing="ij")
    v = np.stack([xs.ravel(), np.zeros(xs.size, np.float32), zs.ravel()], 1)
    idx = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            idx += [[a, b, c], [a, c, d]]
    s = TriangleScene()
    s.add(3, v, np.array(idx, np.uint32))
    quad = np.array([[2, 0, 2], [3, 0, 2], [3, 0, 3], [2, 0, 3]], np.float32)
    s.add(1, quad, np.array([[0, 1, 2], [0, 2, 3]], np.uint32))
    degenerate = np.array([[0.5, 1.0, 0.5], [1.5, 1.0, 0.5], [2.5, 1.0, 0.5]], np.float32)
    s.add(7, degenerate, np.array([[0, 1, 2]], np.uint32))
    return s


def grid_rays(n=8):
    """Rays aimed at grid vertices, edge midpoints and cell centres, straight down, obliquely and along
    axis directions with zero components; plus segment-limit cases."""
    pts = []
    for i in range(n + 1):
        for j in range(n + 1):
            pts += [[i, 0, j], [i + 0.5, 0, j], [i, 0, j + 0.5], [i + 0.5, 0, j + 0.5], [i + 0.25, 0, j + 0.75]]
    pts = np.array(pts, np.float32)
    dirs = [np.array([0, -1, 0], np.float32), np.array([0.3, -1, 0.2], np.float32), np.array([0, -1, 0.5], np.float32)]
    orgs, ds = [], []
    for d in dirs:
        d = d / np.linalg.norm(d)
        orgs.append(pts - 3.0 * d)
        ds.append(np.broadcast_to(d, pts.shape))
    org = np.concatenate(orgs).astype(np.float32)
    dd = np.concatenate(ds).astype(np.float32)
    # grazing rays in the plane of the grid and rays parallel to it just above
    g_org = np.array([[-1, 0, 0.5], [-1, 0, 1.0], [-1, 1e-6, 2.5], [0.5, 0, -1]], np.float32)
    g_dir = np.array([[1, 0, 0], [1, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    targets = np.concatenate([np.tile(pts, (len(dirs), 1)), np.full((4, 3), np.nan, np.float32)])
    return np.concatenate([org, g_org]), np.concatenate([dd, g_dir]), targets


def segment_cases():
    """(org, dir, tnear, tfar) rows straddling the plane y = 0 at t = 3 exactly."""
    org = np.array([[0.5, 3, 0.5]] * 6, np.float32)
    d = np.array([[0, -1, 0]] * 6, np.float32)
    tnear = np.array([0, 0, 0, 3, 3.0000002, 0], np.float32)
    tfar = np.array([np.inf, 3, 2.9999998, 3, np.inf, 0], np.float32)
    return org, d, tnear, tfar


def segment_rayhits():
    org, d, tn, tf = segment_cases()
    r = make_rayhits(org, d)
    r["tnear"], r["tfar"] = tn, tf
    return r


def segment_rays():
    org, d, tn, tf = segment_cases()
    r = make_rays(org, d)
    r["tnear"], r["tfar"] = tn, tf
    return r


def untraceable_rays():
    """Rays no triangle can hit under the watertight test: NaN or infinite origin or direction components,
    a zero direction; each aimed (where finite) at the scene so that a broken guard would show up as hits."""
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    org = np.array([[nan, 40, -170], [0, 40, -170], [inf, 40, -170], [0, 40, -170], [0, -inf, 0], [0, 40, -170],
                    [0, 40, -170]], np.float32)
    d = np.array([[0, 0, 1], [0, nan, 1], [0, 0, 1], [0, 0, inf], [0, 1, 0], [0, 0, 0], [-inf, 0, 1]], np.float32)
    return org, d
