"""Structured meshes with the node/element numbering of the reference's generators.

* `box` follows boxGen (`edelweissfe/generators/boxgen.py:91-330`): grid nodes x outer, y, z
  inner; Hexa20 keeps only nodes with at most one odd grid index (:133-141); Hexa8 / Hexa20
  element node order of :148-299.
* `rect` follows planeRectQuad (`edelweissfe/generators/planerectquad.py:75-143`): nodes x
  outer, y inner; Quad8 centre nodes stay in the node list without DOFs.

DOF numbering is the DofManager's (`numerics/dofmanager.py:259-300`): DOF-carrying nodes in node
order, components interleaved.
"""

import numpy as np

_H8 = [(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)]
_H20 = [
    (0, 0, 0), (0, 0, 2), (2, 0, 2), (2, 0, 0), (0, 2, 0), (0, 2, 2), (2, 2, 2), (2, 2, 0),
    (0, 0, 1), (1, 0, 2), (2, 0, 1), (1, 0, 0), (0, 2, 1), (1, 2, 2), (2, 2, 1), (1, 2, 0),
    (0, 1, 0), (0, 1, 2), (2, 1, 2), (2, 1, 0),
]  # fmt: skip


def box(nX, nY, nZ, lX=1.0, lY=1.0, lZ=1.0, nNodes=8, x0=(0.0, 0.0, 0.0)):
    """coords [n,3], conn [E,nNodes] (int32), nodeDof [n] (int32), nDof."""
    f = 1 if nNodes == 8 else 2
    nx, ny, nz = f * nX + 1, f * nY + 1, f * nZ + 1
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    keep = np.ones(I.size, bool) if nNodes == 8 else (I % 2 + J % 2 + K % 2) < 2
    gid = -np.ones(I.size, np.int64)
    gid[keep] = np.arange(int(keep.sum()))
    gid = gid.reshape(nx, ny, nz)
    xs = np.linspace(x0[0], x0[0] + lX, nx)
    ys = np.linspace(x0[1], x0[1] + lY, ny)
    zs = np.linspace(x0[2], x0[2] + lZ, nz)
    coords = np.stack([xs[I[keep]], ys[J[keep]], zs[K[keep]]], 1)
    ix, iy, iz = np.meshgrid(np.arange(nX), np.arange(nY), np.arange(nZ), indexing="ij")
    ix, iy, iz = f * ix.ravel(), f * iy.ravel(), f * iz.ravel()
    loc = _H8 if nNodes == 8 else _H20
    conn = np.stack([gid[ix + a, iy + b, iz + c] for a, b, c in loc], 1).astype(np.int32)
    n = len(coords)
    return coords, conn, (3 * np.arange(n)).astype(np.int32), 3 * n


def rect(nX, nY, lX=1.0, lY=1.0, nNodes=4, x0=(0.0, 0.0)):
    """coords [n,2], conn [E,nNodes], nodeDof [n] (-1 for Quad8 centre nodes), nDof."""
    f = 1 if nNodes == 4 else 2
    nx, ny = f * nX + 1, f * nY + 1
    g = np.mgrid[x0[0] : x0[0] + lX : nx * 1j, x0[1] : x0[1] + lY : ny * 1j]
    coords = np.stack([g[0].ravel(), g[1].ravel()], 1)
    gid = np.arange(nx * ny).reshape(nx, ny)
    x, y = np.meshgrid(np.arange(nX), np.arange(nY), indexing="ij")
    x, y = f * x.ravel(), f * y.ravel()
    if nNodes == 4:
        loc = [(0, 0), (1, 0), (1, 1), (0, 1)]
    else:
        loc = [(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1)]
    conn = np.stack([gid[x + a, y + b] for a, b in loc], 1).astype(np.int32)
    used = np.zeros(len(coords), bool)
    used[conn.ravel()] = True
    nodeDof = -np.ones(len(coords), np.int32)
    nodeDof[used] = 2 * np.arange(int(used.sum()))
    return coords, conn, nodeDof, 2 * int(used.sum())


def jitter(coords, frac, h, seed, lo, hi):
    """Move nodes strictly inside [lo, hi] by U(-frac, frac) * h per axis (seeded)."""
    rng = np.random.default_rng(seed)
    coords = coords.copy()
    inside = np.all((coords > np.asarray(lo) + 1e-9) & (coords < np.asarray(hi) - 1e-9), axis=1)
    coords[inside] += rng.uniform(-frac, frac, (int(inside.sum()), coords.shape[1])) * np.asarray(h)
    return coords
