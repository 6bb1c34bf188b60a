"""Seeded synthetic problems in the reference's assembled format.

No public benchmark suite exists for this path, so every workload is
generated here from a seed:

* ``poisson2d_p1`` -- -Laplace(u) = f on the unit square with P1 triangles on a
  jittered node grid, each cell split along a random diagonal, homogeneous
  Dirichlet boundary (boundary nodes removed), f ~ U[-1, 1] per node with a
  mass-lumped load.  129 x 129 nodes give 16,129 unknowns.
* ``diffusion3d_fv`` -- -div(kappa grad u) = f on a cell-centred N^3 grid, 7-point
  finite volumes with harmonic-mean face coefficients, Dirichlet boundary,
  kappa = exp(g) with g a Gaussian field (std sigma, correlation length `corr`
  cells, FFT-filtered white noise), f ~ U[-1, 1].  N = 128 gives 2,097,152
  unknowns and 14,581,760 nonzeros.
* ``block_partition`` -- the stand-in for a METIS partition of a structured
  grid: equal boxes of cells, numbered 1..nparts.
* ``poisson2d_p1_elements`` -- the same 2-D P1 problem as element matrices
  (DOUG's elemental input, input_type 1), optionally with one conductivity
  per element; ``write_elemental_files`` writes them in DOUG's files.

Matrices are returned as 1-based COO triplets sorted by row then column, as
an assembled text file would list them.
"""
from __future__ import annotations

import numpy as np


def _csr_to_coo1(A):
    A = A.tocsr()
    A.sort_indices()
    rows = np.repeat(np.arange(A.shape[0], dtype=np.int64), np.diff(A.indptr))
    return (rows + 1).astype(np.int32), (A.indices + 1).astype(np.int32), A.data.astype(np.float64)


def poisson2d_p1(nodes: int = 129, jitter: float = 0.2, seed: int = 0):
    """Returns (n, rows1, cols1, vals, rhs, coords) for the 2-D P1 problem."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    h = 1.0 / (nodes - 1)
    ii, jj = np.meshgrid(np.arange(nodes), np.arange(nodes), indexing="ij")
    x = ii * h
    y = jj * h
    interior = (ii > 0) & (ii < nodes - 1) & (jj > 0) & (jj < nodes - 1)
    dx = rng.uniform(-jitter * h, jitter * h, size=x.shape)
    dy = rng.uniform(-jitter * h, jitter * h, size=y.shape)
    x = np.where(interior, x + dx, x)
    y = np.where(interior, y + dy, y)
    gid = ii * nodes + jj
    X = x.ravel()
    Y = y.ravel()
    c0 = gid[:-1, :-1].ravel()
    c1 = gid[1:, :-1].ravel()
    c2 = gid[1:, 1:].ravel()
    c3 = gid[:-1, 1:].ravel()
    diag = rng.integers(0, 2, size=c0.shape)  # which diagonal splits the cell
    t1 = np.where(diag[:, None] == 0, np.stack([c0, c1, c2], 1), np.stack([c0, c1, c3], 1))
    t2 = np.where(diag[:, None] == 0, np.stack([c0, c2, c3], 1), np.stack([c1, c2, c3], 1))
    tri = np.concatenate([t1, t2], 0)
    px = X[tri]
    py = Y[tri]
    b = np.stack([py[:, 1] - py[:, 2], py[:, 2] - py[:, 0], py[:, 0] - py[:, 1]], 1)
    c = np.stack([px[:, 2] - px[:, 1], px[:, 0] - px[:, 2], px[:, 1] - px[:, 0]], 1)
    area = 0.5 * (px[:, 1] * py[:, 2] - px[:, 2] * py[:, 1] - px[:, 0] * py[:, 2]
                  + px[:, 2] * py[:, 0] + px[:, 0] * py[:, 1] - px[:, 1] * py[:, 0])
    area = np.abs(area)
    K = (b[:, :, None] * b[:, None, :] + c[:, :, None] * c[:, None, :]) / (4.0 * area[:, None, None])
    R = np.repeat(tri, 3, axis=1).ravel()
    Cc = np.tile(tri, (1, 3)).ravel()
    A = sp.coo_matrix((K.ravel(), (R, Cc)), shape=(nodes * nodes,) * 2).tocsr()
    f = rng.uniform(-1.0, 1.0, size=nodes * nodes)
    lump = np.zeros(nodes * nodes)
    np.add.at(lump, tri.ravel(), np.repeat(area / 3.0, 3))
    load = f * lump
    keep = np.flatnonzero(interior.ravel())
    A = A[keep][:, keep]
    rows1, cols1, vals = _csr_to_coo1(A)
    coords = np.stack([X[keep], Y[keep]], 1)
    return len(keep), rows1, cols1, vals, load[keep].copy(), coords


def batched_poisson2d_p1(nsys: int = 256, n_min: int = 2000, n_max: int = 200000, seed: int = 0):
    """Uneven independent systems: ``nsys`` jittered P1 Poisson problems as
    poisson2d_p1, unknown counts drawn log-uniform in [n_min, n_max] (each
    rounded to a square grid of interior nodes), each with its own seeded
    jitter, diagonals and load.  Returns a list of (n, rows1, cols1, vals, rhs)."""
    rng = np.random.default_rng(seed)
    target = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=nsys))
    out = []
    for k, t in enumerate(target):
        nodes = int(round(np.sqrt(t))) + 2
        n, r, c, v, b, _ = poisson2d_p1(nodes, seed=seed * 100003 + k + 1)
        out.append((n, r, c, v, b))
    return out


def poisson2d_p1_elements(nodes: int = 17, jitter: float = 0.2, seed: int = 0, kappa=None):
    """The P1 problem of ``poisson2d_p1`` as element matrices.

    Freedoms are the interior nodes (numbered 1..ngf in node order; boundary
    nodes carry no freedom, as in DOUG's freemap); element e lists its interior
    vertices.  kappa (one value per triangle, default 1) scales the element
    stiffness.  Returns (ngf, eptr, efree, emat, erhs, info) with emat the
    element matrices column by column and info a dict of the mesh sizes,
    the node coordinates info["coords"] (nnode x 2) and the node of every
    freedom info["freemap"] (1-based).
    """
    rng = np.random.default_rng(seed)
    h = 1.0 / (nodes - 1)
    ii, jj = np.meshgrid(np.arange(nodes), np.arange(nodes), indexing="ij")
    x = ii * h
    y = jj * h
    interior = (ii > 0) & (ii < nodes - 1) & (jj > 0) & (jj < nodes - 1)
    dx = rng.uniform(-jitter * h, jitter * h, size=x.shape)
    dy = rng.uniform(-jitter * h, jitter * h, size=y.shape)
    x = np.where(interior, x + dx, x)
    y = np.where(interior, y + dy, y)
    gid = ii * nodes + jj
    X = x.ravel()
    Y = y.ravel()
    c0 = gid[:-1, :-1].ravel()
    c1 = gid[1:, :-1].ravel()
    c2 = gid[1:, 1:].ravel()
    c3 = gid[:-1, 1:].ravel()
    diag = rng.integers(0, 2, size=c0.shape)
    t1 = np.where(diag[:, None] == 0, np.stack([c0, c1, c2], 1), np.stack([c0, c1, c3], 1))
    t2 = np.where(diag[:, None] == 0, np.stack([c0, c2, c3], 1), np.stack([c1, c2, c3], 1))
    tri = np.concatenate([t1, t2], 0)
    px = X[tri]
    py = Y[tri]
    b = np.stack([py[:, 1] - py[:, 2], py[:, 2] - py[:, 0], py[:, 0] - py[:, 1]], 1)
    c = np.stack([px[:, 2] - px[:, 1], px[:, 0] - px[:, 2], px[:, 1] - px[:, 0]], 1)
    area = np.abs(0.5 * (px[:, 1] * py[:, 2] - px[:, 2] * py[:, 1] - px[:, 0] * py[:, 2]
                         + px[:, 2] * py[:, 0] + px[:, 0] * py[:, 1] - px[:, 1] * py[:, 0]))
    K = (b[:, :, None] * b[:, None, :] + c[:, :, None] * c[:, None, :]) / (4.0 * area[:, None, None])
    if kappa is not None:
        K = K * np.asarray(kappa, dtype=np.float64)[:, None, None]
    f = rng.uniform(-1.0, 1.0, size=nodes * nodes)
    free = np.zeros(nodes * nodes, dtype=np.int64)
    free[interior.ravel()] = np.arange(1, int(interior.sum()) + 1)
    ft = free[tri]                                    # (ne, 3), 0 = boundary vertex
    mask = ft > 0
    eptr = np.concatenate([[0], np.cumsum(mask.sum(1))]).astype(np.int32)
    efree = ft[mask].astype(np.int32)
    m2 = mask[:, :, None] & mask[:, None, :]          # (e, j, i): column j, row i
    emat = np.ascontiguousarray(K.transpose(0, 2, 1))[m2]      # column by column
    erhs = (f[tri] * area[:, None] / 3.0)[mask]
    info = {"nell": len(tri), "ngf": int(interior.sum()), "nsd": 2, "mfrelt": 3, "nnode": nodes * nodes,
            "coords": np.stack([X, Y], 1), "freemap": (np.flatnonzero(interior.ravel()) + 1).astype(np.int32)}
    return info["ngf"], eptr, efree, np.asarray(emat, np.float64), np.asarray(erhs, np.float64), info


def _kuhn_tets(N: int):
    """Node ids of the 6 Kuhn tetrahedra of every hex of an N^3 grid of
    (N+1)^3 nodes (node id (i*(N+1) + j)*(N+1) + k; conforming across hexes)."""
    n1 = N + 1
    I, J, K = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    base = ((I * n1 + J) * n1 + K).ravel()
    step = np.array([n1 * n1, n1, 1])
    tets = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        a = step[perm[0]]
        b = a + step[perm[1]]
        c = b + step[perm[2]]
        tets.append(np.stack([base, base + a, base + b, base + c], 1))
    return np.concatenate(tets, 0)


def elasticity3d_p1_elements(N: int = 64, jitter: float = 0.15, nboxes: int = 20, e_box: float = 1.0e3,
                             nu: float = 0.3, seed: int = 0):
    """3-D linear elasticity on P1 tetrahedra (element input, 3 freedoms per node).

    The unit cube is an N^3 hex grid, every hex split into 6 Kuhn tetrahedra,
    nodes off the boundary jittered uniformly by +-jitter*h (seeded).  Young's
    modulus 1, except E = e_box in elements whose centroid lies in one of
    ``nboxes`` seeded axis-aligned boxes; Poisson ratio nu.  The bottom face
    (z = 0) is clamped (its freedoms are left out, as DOUG's freemap does);
    body force (0, 0, -1) lumped to the vertices.  Freedom of node n (z > 0),
    component c: 3*(index of n among the free nodes) + c + 1.

    Returns (ngf, eptr, efree, emat, erhs, info) in the layout of
    ``poisson2d_p1_elements`` (element matrices column by column, restricted
    to the element's free freedoms), plus info["node_ijk"] (free node grid
    indices, for box partitions), info["coords"] (nnode x 3) and
    info["freemap"] (the 1-based node of every freedom).
    """
    rng = np.random.default_rng(seed)
    n1 = N + 1
    h = 1.0 / N
    I, J, K = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    X = np.stack([I, J, K], -1).reshape(-1, 3) * h
    inner = ((I > 0) & (I < N) & (J > 0) & (J < N) & (K > 0) & (K < N)).ravel()
    X[inner] += rng.uniform(-jitter * h, jitter * h, size=(int(inner.sum()), 3))
    tet = _kuhn_tets(N)
    P = X[tet]                                          # (ne, 4, 3)
    Jm = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], 2)   # columns = edges
    det = np.linalg.det(Jm)
    vol = np.abs(det) / 6.0
    Ji = np.linalg.inv(Jm)                              # rows: gradients of the barycentric coords 1..3
    grad = np.concatenate([-Ji.sum(1, keepdims=True), Ji], 1)                  # (ne, 4, 3)
    ne = tet.shape[0]
    B = np.zeros((ne, 6, 12))
    for a in range(4):
        gx, gy, gz = grad[:, a, 0], grad[:, a, 1], grad[:, a, 2]
        c = 3 * a
        B[:, 0, c] = gx
        B[:, 1, c + 1] = gy
        B[:, 2, c + 2] = gz
        B[:, 3, c] = gy
        B[:, 3, c + 1] = gx
        B[:, 4, c + 1] = gz
        B[:, 4, c + 2] = gy
        B[:, 5, c] = gz
        B[:, 5, c + 2] = gx
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[[0, 1, 2], [0, 1, 2]] = lam + 2 * mu
    D[[3, 4, 5], [3, 4, 5]] = mu
    lo = rng.uniform(0.0, 0.85, size=(nboxes, 3))
    hi = lo + rng.uniform(0.05, 0.25, size=(nboxes, 3))
    cen = P.mean(1)
    inbox = np.zeros(ne, dtype=bool)
    for q in range(nboxes):
        inbox |= np.all((cen >= lo[q]) & (cen <= hi[q]), axis=1)
    E = np.where(inbox, e_box, 1.0)
    Ke = np.matmul(np.matmul(B.transpose(0, 2, 1), D), B) * (E * vol)[:, None, None]   # (ne, 12, 12)
    Ke = 0.5 * (Ke + Ke.transpose(0, 2, 1))            # symmetric to the last bit
    del B
    # freedoms: nodes with k > 0
    kz = K.ravel()
    freenode = np.full(n1 ** 3, -1, dtype=np.int64)
    freenode[kz > 0] = np.arange(int((kz > 0).sum()))
    ngf = 3 * int((kz > 0).sum())
    dof = (3 * freenode[tet])[:, :, None] + np.arange(3)[None, None, :] + 1        # (ne, 4, 3), 1-based
    dof = np.where((freenode[tet] >= 0)[:, :, None], dof, 0).reshape(ne, 12)
    mask = dof > 0
    nf = mask.sum(1)
    eptr = np.concatenate([[0], np.cumsum(nf)]).astype(np.int32)
    efree = dof[mask].astype(np.int32)
    m2 = mask[:, :, None] & mask[:, None, :]            # (e, j, i): column j, row i
    emat = np.ascontiguousarray(Ke.transpose(0, 2, 1))[m2]
    load = np.zeros((ne, 4, 3))
    load[:, :, 2] = -(vol / 4.0)[:, None]
    erhs = load.reshape(ne, 12)[mask]
    fn = np.flatnonzero(kz > 0)
    info = {"nell": ne, "ngf": ngf, "nsd": 3, "mfrelt": 12, "nnode": n1 ** 3,
            "node_ijk": np.stack([I.ravel()[fn], J.ravel()[fn], kz[fn]], 1),
            "coords": X, "freemap": (np.repeat(fn, 3) + 1).astype(np.int32)}
    return ngf, eptr, efree, emat, erhs, info


def dof_box_partition(node_ijk, N: int, parts=(4, 4, 8), dofs_per_node: int = 3):
    """1-based box-partition ids of the freedoms (``dofs_per_node`` per node)
    from the free nodes' grid indices (i, j in 0..N, k in 1..N)."""
    i, j, k = node_ijk[:, 0], node_ijk[:, 1], node_ijk[:, 2] - 1
    bi = np.minimum(i * parts[0] // (N + 1), parts[0] - 1)
    bj = np.minimum(j * parts[1] // (N + 1), parts[1] - 1)
    bk = np.minimum(k * parts[2] // N, parts[2] - 1)
    p = (bi * parts[1] + bj) * parts[2] + bk
    return (np.repeat(p, dofs_per_node) + 1).astype(np.int32)


def _fortran_record(fh, payload: bytes) -> None:
    n = np.array([len(payload)], dtype="<i4").tobytes()
    fh.write(n + payload + n)


def write_elemental_files(folder: str, ngf, eptr, efree, emat, erhs, info) -> dict:
    """Writes DOUG's elemental input files (Fortran unformatted sequential,
    little-endian): info, freedom lists and element matrices + RHS, and when
    info has "coords" and "freemap" the node coordinates (one record,
    coordinate after coordinate of every node) and the freedom-to-node map
    (one record).  Returns the control-file words that name them."""
    import os
    eptr = np.asarray(eptr)
    files = {"info_file": "doug_info.dat", "freedom_lists_file": "doug_element.dat",
             "elemmat_rhs_file": "doug_system.dat"}
    with open(os.path.join(folder, files["info_file"]), "wb") as fh:
        _fortran_record(fh, np.array([info["nell"], ngf, info["nsd"], info["mfrelt"], info["nnode"]],
                                     dtype="<i4").tobytes())
    with open(os.path.join(folder, files["freedom_lists_file"]), "wb") as fh:
        for e in range(len(eptr) - 1):
            fr = np.asarray(efree[eptr[e]:eptr[e + 1]], dtype="<i4")
            _fortran_record(fh, np.array([len(fr)], dtype="<i4").tobytes() + fr.tobytes())
    with open(os.path.join(folder, files["elemmat_rhs_file"]), "wb") as fh:
        off = 0
        for e in range(len(eptr) - 1):
            nf = int(eptr[e + 1] - eptr[e])
            for j in range(nf):
                _fortran_record(fh, np.asarray(emat[off + j * nf: off + (j + 1) * nf], dtype="<f8").tobytes())
            off += nf * nf
            _fortran_record(fh, np.asarray(erhs[eptr[e]:eptr[e + 1]], dtype="<f8").tobytes())
    if "coords" in info and "freemap" in info:
        files["coords_file"] = "doug_coord.dat"
        files["freemap_file"] = "doug_freemap.dat"
        with open(os.path.join(folder, files["coords_file"]), "wb") as fh:
            _fortran_record(fh, np.ascontiguousarray(info["coords"], dtype="<f8").tobytes())
        with open(os.path.join(folder, files["freemap_file"]), "wb") as fh:
            _fortran_record(fh, np.ascontiguousarray(info["freemap"], dtype="<i4").tobytes())
    return files


def gaussian_field_3d(N: int, sigma: float = 1.0, corr: float = 8.0, seed: int = 0):
    """Stationary Gaussian field: FFT-filtered white noise with a Gaussian
    covariance of correlation length `corr` cells, scaled to std `sigma`."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((N, N, N))
    k = np.fft.fftfreq(N) * 2.0 * np.pi
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    filt = np.exp(-0.25 * (corr ** 2) * (kx ** 2 + ky ** 2 + kz ** 2))
    g = np.real(np.fft.ifftn(np.fft.fftn(w) * filt))
    g -= g.mean()
    g *= sigma / g.std()
    return g


def diffusion3d_fv(N: int = 128, sigma: float = 1.0, corr: float = 8.0, seed: int = 0):
    """Returns (n, rows1, cols1, vals, rhs) of the cell-centred 7-point problem."""
    g = gaussian_field_3d(N, sigma, corr, seed)
    kap = np.exp(g)
    rng = np.random.default_rng(seed + 1)
    f = rng.uniform(-1.0, 1.0, size=N ** 3)
    idx = np.arange(N ** 3, dtype=np.int64).reshape(N, N, N)
    diag = np.zeros((N, N, N))
    rows, cols, vals = [], [], []
    for ax in range(3):
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[ax] = slice(0, N - 1)
        b[ax] = slice(1, N)
        ka = kap[tuple(a)]
        kb = kap[tuple(b)]
        t = 2.0 * ka * kb / (ka + kb)           # harmonic mean face coefficient
        diag[tuple(a)] += t
        diag[tuple(b)] += t
        ia = idx[tuple(a)].ravel()
        ib = idx[tuple(b)].ravel()
        rows += [ia, ib]
        cols += [ib, ia]
        vals += [-t.ravel(), -t.ravel()]
        # Dirichlet faces: half-cell distance gives 2 kappa
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = 0
        hi[ax] = N - 1
        diag[tuple(lo)] += 2.0 * kap[tuple(lo)]
        diag[tuple(hi)] += 2.0 * kap[tuple(hi)]
    rows.append(idx.ravel())
    cols.append(idx.ravel())
    vals.append(diag.ravel())
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = np.concatenate(vals)
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    return N ** 3, (r + 1).astype(np.int32), (c + 1).astype(np.int32), v, f


def block_partition(N: int, parts_per_dim: int, dim: int = 3):
    """1-based ids of equal boxes of an N^dim grid (row-major cell order)."""
    b = np.arange(N) * parts_per_dim // N
    if dim == 2:
        I, J = np.meshgrid(b, b, indexing="ij")
        p = I * parts_per_dim + J
    else:
        I, J, K = np.meshgrid(b, b, b, indexing="ij")
        p = (I * parts_per_dim + J) * parts_per_dim + K
    return (p.ravel() + 1).astype(np.int32)


def laplace2d(m: int):
    """5-point Laplacian on an m x m grid (the reference's LapNxN fixtures)."""
    n = m * m
    r, c, v = [], [], []
    for i in range(m):
        for j in range(m):
            k = i * m + j
            r.append(k); c.append(k); v.append(4.0)
            for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                a, b = i + di, j + dj
                if 0 <= a < m and 0 <= b < m:
                    r.append(k); c.append(a * m + b); v.append(-1.0)
    return n, np.array(r, np.int32) + 1, np.array(c, np.int32) + 1, np.array(v), np.ones(n)
