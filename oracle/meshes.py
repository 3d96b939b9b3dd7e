"""Structured meshes with the reference generators' node and element numbering.

* planeRectQuad (`edelweissfe/generators/planerectquad.py:75-200`): nodes on an
  mgrid, x outer / y inner; Quad4 and Quad8 connectivity; Quad8 centre nodes
  stay in the node list but carry no DOFs (nodefield.py:86).
* boxGen (`edelweissfe/generators/boxgen.py:91-330`): nodes x outer, y, z inner;
  Hexa20 skips nodes with two or more odd grid indices (:133-141).

DOF numbering follows DofManager (dofmanager.py:259-300): nodes that carry the
displacement field, in node order, ``dof = 2*pos`` (2D) / ``3*pos`` (3D) + component.
"""

import numpy as np


def plane_rect_quad(nX, nY, l=1.0, h=1.0, x0=0.0, y0=0.0, nNodes=4):  # noqa: E741
    """Returns coords [nAll,2], conn [E,nN] into coords, node_dof [nAll] (-1 = no DOF), nDof."""
    if nNodes == 4:
        nx, ny = nX + 1, nY + 1
    else:
        nx, ny = 2 * nX + 1, 2 * nY + 1
    grid = np.mgrid[x0 : x0 + l : nx * 1j, y0 : y0 + h : ny * 1j]  # planerectquad.py:100-103
    coords = np.stack([grid[0].reshape(-1), grid[1].reshape(-1)], axis=1)  # x outer, y inner
    gid = np.arange(nx * ny).reshape(nx, ny)
    conn = []
    for x in range(nX):
        for y in range(nY):
            if nNodes == 4:
                conn.append([gid[x, y], gid[x + 1, y], gid[x + 1, y + 1], gid[x, y + 1]])
            else:
                conn.append(
                    [
                        gid[2 * x, 2 * y],
                        gid[2 * x + 2, 2 * y],
                        gid[2 * x + 2, 2 * y + 2],
                        gid[2 * x, 2 * y + 2],
                        gid[2 * x + 1, 2 * y],
                        gid[2 * x + 2, 2 * y + 1],
                        gid[2 * x + 1, 2 * y + 2],
                        gid[2 * x, 2 * y + 1],
                    ]
                )
    conn = np.array(conn, np.int64)
    used = np.zeros(len(coords), bool)
    used[conn.reshape(-1)] = True
    node_dof = -np.ones(len(coords), np.int64)
    node_dof[used] = 2 * np.arange(used.sum())
    return coords, conn, node_dof, int(2 * used.sum())


def box_gen(nX, nY, nZ, lX=1.0, lY=1.0, lZ=1.0, x0=0.0, y0=0.0, z0=0.0, nNodes=8):
    """Returns coords [nUsed,3], conn [E,nN], node_dof [nUsed], nDof (boxgen.py:91-330)."""
    if nNodes == 8:
        nx, ny, nz = nX + 1, nY + 1, nZ + 1
    else:
        nx, ny, nz = 2 * nX + 1, 2 * nY + 1, 2 * nZ + 1
    xs = np.linspace(x0, x0 + lX, nx)
    ys = np.linspace(y0, y0 + lY, ny)
    zs = np.linspace(z0, z0 + lZ, nz)
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    if nNodes == 8:
        keep = np.ones(len(I), bool)
    else:
        keep = (I % 2 + J % 2 + K % 2) < 2
    gid = -np.ones(nx * ny * nz, np.int64)
    gid[keep] = np.arange(keep.sum())
    gid = gid.reshape(nx, ny, nz)
    coords = np.stack([xs[I[keep]], ys[J[keep]], zs[K[keep]]], axis=1)
    ix, iy, iz = np.meshgrid(np.arange(nX), np.arange(nY), np.arange(nZ), indexing="ij")
    ix, iy, iz = ix.reshape(-1), iy.reshape(-1), iz.reshape(-1)
    if nNodes == 8:
        loc = [(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)]
        conn = np.stack([gid[ix + a, iy + b, iz + c] for a, b, c in loc], axis=1)
    else:
        loc = [
            (0, 0, 0), (0, 0, 2), (2, 0, 2), (2, 0, 0), (0, 2, 0), (0, 2, 2), (2, 2, 2), (2, 2, 0),
            (0, 0, 1), (1, 0, 2), (2, 0, 1), (1, 0, 0), (0, 2, 1), (1, 2, 2), (2, 2, 1), (1, 2, 0),
            (0, 1, 0), (0, 1, 2), (2, 1, 2), (2, 1, 0),
        ]  # fmt: skip
        conn = np.stack([gid[2 * ix + a, 2 * iy + b, 2 * iz + c] for a, b, c in loc], axis=1)
    node_dof = 3 * np.arange(len(coords), dtype=np.int64)
    return coords, conn.astype(np.int64), node_dof, 3 * len(coords)


def jitter_interior(coords, frac, h, rng, lo, hi):
    """Move nodes strictly inside the box [lo, hi] by U(-frac, frac) * h per axis."""
    coords = coords.copy()
    inside = np.all((coords > np.asarray(lo) + 1e-9) & (coords < np.asarray(hi) - 1e-9), axis=1)
    coords[inside] += rng.uniform(-frac, frac, (inside.sum(), coords.shape[1])) * np.asarray(h)
    return coords
