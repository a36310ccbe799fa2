"""Seeded hex box meshes in the reference's native layout, in numpy.

The same mesh as the library's generator fc_mesh_box (hexes only): vertex
(i, j, k) at (i hx, j hy, k hz), interior vertices moved by
(2u - 1) * perturb * h per axis with u from splitmix64 in x, y, z order; inner
faces per cell in (+x, +y, +z) order, so sorted by (owner, neighbour); the
six boundary patches xmin, xmax, ymin, ymax, zmin, zmax with outward node
order.  It lets the CPU arm of the benchmark and the tests build the
oracle's inputs without loading the GPU library; tests/test_box_mesh.py
checks it against fc_mesh_box array for array.
"""
import numpy as np

NOMAX = 6
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64_uniform(seed, count):
    """The first `count` draws of splitmix64(seed) as doubles in [0, 1)
    with 53 random bits."""
    k = np.arange(1, count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _vertices(nx, ny, nz, lx, ly, lz, perturb, seed):
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    x, y, z = i * hx, j * hy, k * hz
    if perturb > 0:
        inner = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
        m = int(inner.sum())
        u = splitmix64_uniform(seed, 3 * m).reshape(m, 3)
        x = x.astype(np.float64)
        y = y.astype(np.float64)
        z = z.astype(np.float64)
        x[inner] += (2.0 * u[:, 0] - 1.0) * perturb * hx
        y[inner] += (2.0 * u[:, 1] - 1.0) * perturb * hy
        z[inner] += (2.0 * u[:, 2] - 1.0) * perturb * hz
    return x.astype(np.float64), y.astype(np.float64), z.astype(np.float64)


def hex_box(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, perturb=0.0, seed=42, bctype=None):
    """Arrays dict of the box mesh (1-based indices), the layout that
    oracle_lib.Case and fcgpu.Mesh.from_arrays take."""
    x, y, z = _vertices(nx, ny, nz, lx, ly, lz, perturb, seed)

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k) + 1

    def cid(i, j, k):
        return i + nx * (j + ny * k) + 1

    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    c = cid(i, j, k)
    # per cell, up to three inner faces in +x, +y, +z order
    quads = np.zeros((len(c), 3, 4), np.int64)
    own = np.zeros((len(c), 3), np.int64)
    nbr = np.zeros((len(c), 3), np.int64)
    has = np.zeros((len(c), 3), bool)
    has[:, 0] = i + 1 < nx
    quads[:, 0] = np.stack([nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i + 1, j + 1, k + 1), nid(i + 1, j, k + 1)], 1)
    nbr[:, 0] = cid(i + 1, j, k)
    has[:, 1] = j + 1 < ny
    quads[:, 1] = np.stack([nid(i, j + 1, k), nid(i, j + 1, k + 1), nid(i + 1, j + 1, k + 1), nid(i + 1, j + 1, k)], 1)
    nbr[:, 1] = cid(i, j + 1, k)
    has[:, 2] = k + 1 < nz
    quads[:, 2] = np.stack([nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)], 1)
    nbr[:, 2] = cid(i, j, k + 1)
    own[:] = c[:, None]
    sel = has.ravel()
    f_nodes = [quads.reshape(-1, 4)[sel]]
    f_own = [own.ravel()[sel]]
    neighbour = nbr.ravel()[sel]
    nfaces, start = [], []
    n_inner = len(neighbour)
    cur = n_inner

    def patch(nodes4, owner):
        nonlocal cur
        f_nodes.append(np.stack(nodes4, 1).reshape(-1, 4))
        f_own.append(np.asarray(owner).ravel())
        start.append(cur)
        nfaces.append(len(f_own[-1]))
        cur += nfaces[-1]

    kk, jj = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij")
    kk, jj = kk.ravel(), jj.ravel()
    patch([nid(0, jj, kk), nid(0, jj, kk + 1), nid(0, jj + 1, kk + 1), nid(0, jj + 1, kk)], cid(0, jj, kk))
    patch([nid(nx, jj, kk), nid(nx, jj + 1, kk), nid(nx, jj + 1, kk + 1), nid(nx, jj, kk + 1)], cid(nx - 1, jj, kk))
    kk, ii = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    kk, ii = kk.ravel(), ii.ravel()
    patch([nid(ii, 0, kk), nid(ii + 1, 0, kk), nid(ii + 1, 0, kk + 1), nid(ii, 0, kk + 1)], cid(ii, 0, kk))
    patch([nid(ii, ny, kk), nid(ii, ny, kk + 1), nid(ii + 1, ny, kk + 1), nid(ii + 1, ny, kk)], cid(ii, ny - 1, kk))
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    jj, ii = jj.ravel(), ii.ravel()
    patch([nid(ii, jj, 0), nid(ii, jj + 1, 0), nid(ii + 1, jj + 1, 0), nid(ii + 1, jj, 0)], cid(ii, jj, 0))
    patch([nid(ii, jj, nz), nid(ii + 1, jj, nz), nid(ii + 1, jj + 1, nz), nid(ii, jj + 1, nz)], cid(ii, jj, nz - 1))
    q = np.concatenate(f_nodes)
    nF = len(q)
    nodes = np.zeros((nF, NOMAX), np.int32)
    nodes[:, :4] = q
    numCells = nx * ny * nz
    return dict(x=x, y=y, z=z, nnodes=np.full(nF, 4, np.int32), nodes=nodes.ravel(),
                owner=np.concatenate(f_own).astype(np.int32), neighbour=neighbour.astype(np.int32),
                bctype=np.asarray(bctype if bctype is not None else [1] * 6, np.int32),
                nfaces=np.asarray(nfaces, np.int32), startFace=np.asarray(start, np.int32),
                numNodes=len(x), numCells=numCells, numInnerFaces=n_inner, numBoundaryFaces=nF - n_inner)
