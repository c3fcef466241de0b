"""The reference's ghosted array layouts (src/bluebottle.h:70-73) for dense
arrays, one rank, DOM_BUF = 1.  Cells: GCC_LOC = i + j s1b + k s2b over
(nx+2)(ny+2)(nz+2).  Faces: GFX_LOC = j + k s1b + i s2b (x-faces, nx+1 of them
per row), GFY_LOC = k + i s1b + j s2b, GFZ_LOC = i + j s1b + k s2b.  Dense
arrays are (nz, ny, nx) for cells and (nz, ny, nx+1), (nz, ny+1, nx),
(nz+1, ny, nx) for the faces, x fastest."""
import numpy as np


def cells_to_s3b(a):
    nz, ny, nx = a.shape
    b = np.zeros((nz + 2, ny + 2, nx + 2))
    b[1:-1, 1:-1, 1:-1] = a
    return b.ravel()


def cells_from_s3b(b, dims):
    nx, ny, nz = dims
    return b.reshape(nz + 2, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1].copy()


# face arrays: the s3b array as [slowest][middle][fastest] of its own order
def fx_to_s3b(u):
    nz, ny, nx1 = u.shape  # GFX: i slowest (nx+3), then k (nz+2), j fastest (ny+2)
    b = np.zeros((nx1 + 2, nz + 2, ny + 2))
    b[1:-1, 1:-1, 1:-1] = u.transpose(2, 0, 1)
    return b.ravel()


def fx_from_s3b(b, dims):
    nx, ny, nz = dims
    return b.reshape(nx + 3, nz + 2, ny + 2)[1:-1, 1:-1, 1:-1].transpose(1, 2, 0).copy()


def fy_to_s3b(v):
    nz, ny1, nx = v.shape  # GFY: j slowest (ny+3), then i (nx+2), k fastest (nz+2)
    b = np.zeros((ny1 + 2, nx + 2, nz + 2))
    b[1:-1, 1:-1, 1:-1] = v.transpose(1, 2, 0)
    return b.ravel()


def fy_from_s3b(b, dims):
    nx, ny, nz = dims
    return b.reshape(ny + 3, nx + 2, nz + 2)[1:-1, 1:-1, 1:-1].transpose(2, 0, 1).copy()


def fz_to_s3b(w):
    nz1, ny, nx = w.shape  # GFZ: k slowest (nz+3), then j (ny+2), i fastest (nx+2)
    b = np.zeros((nz1 + 2, ny + 2, nx + 2))
    b[1:-1, 1:-1, 1:-1] = w
    return b.ravel()


def fz_from_s3b(b, dims):
    nx, ny, nz = dims
    return b.reshape(nz + 3, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1].copy()
