"""Synthetic subdomain data generators for the BDDC interface solve.

These build, per subdomain, exactly the arrays a caller of the
``bddcml_upload_subdomain_data_c`` entry point hands over: element
connectivity, local-to-global node/dof/element maps, coordinates, Dirichlet
flags and values, the right-hand side, the initial guess and the upper-triangle
COO triplets of the subdomain stiffness matrix.

The Poisson generator restates the reference example program
``examples/poisson_on_cube.f90``:

* element matrix of the Q1 Laplacian on the reference cube, scaled by the
  element size h (``poisson_on_cube.f90:169-177`` and ``:447``);
* lexicographic node numbering inside a subdomain, x fastest
  (``poisson_on_cube.f90:778-826``), element node order n1..n8 (``:836-870``);
* homogeneous Dirichlet condition on the whole boundary of the unit cube
  (``:812-820``);
* right-hand side h^3 at every node, zero at fixed nodes, marked complete so
  that interface weights are applied to it (``:433-437``);
* upper-triangle triplets element by element, unassembled
  (``:449-475``).

A per-element coefficient ``kappa`` multiplies each element matrix; it is 1 in
the reference example and random for the heterogeneous workloads.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional

import numpy as np

# Q1 Laplacian element matrix on [0,1]^3 with the node order of the reference
# example (n1=(0,0,0), n2=(1,0,0), n3=(1,1,0), n4=(0,1,0), n5..n8 = +z).
# Entries: 1/3 on the diagonal, 0 for nodes differing in one coordinate,
# -1/12 for nodes differing in two or three coordinates.
_NODE_OFFSETS = np.array(
    [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
     [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.int64)


def q1_laplace_reference_matrix() -> np.ndarray:
    km = np.zeros((8, 8))
    for i in range(8):
        for j in range(8):
            d = int(np.abs(_NODE_OFFSETS[i] - _NODE_OFFSETS[j]).sum())
            if d == 0:
                km[i, j] = 1.0 / 3.0
            elif d == 1:
                km[i, j] = 0.0
            else:
                km[i, j] = -1.0 / 12.0
    return km


@dataclasses.dataclass
class Subdomain:
    """Arrays of one subdomain, 0-based (numbase = 0)."""
    isub: int
    nelems: int
    nnods: int
    ndofs: int
    inet: np.ndarray      # int32, nelems*8
    nnet: np.ndarray      # int32, nelems
    nndf: np.ndarray      # int32, nnods
    isngn: np.ndarray     # int32, nnods
    isvgvn: np.ndarray    # int32, ndofs
    isegn: np.ndarray     # int32, nelems
    xyz: np.ndarray       # float64, (ndim, nnods) column-major as Fortran xyz(lxyz1,lxyz2)
    ifix: np.ndarray      # int32, ndofs
    fixv: np.ndarray      # float64, ndofs
    rhs: np.ndarray       # float64, ndofs
    sol: np.ndarray       # float64, ndofs
    i_sparse: np.ndarray  # int32, la
    j_sparse: np.ndarray  # int32, la
    a_sparse: np.ndarray  # float64, la
    is_rhs_complete: int = 1
    is_assembled: int = 0


@dataclasses.dataclass
class Problem:
    name: str
    nelem: int
    nnod: int
    ndof: int
    ndim: int
    meshdim: int
    subdomains: List[Subdomain]
    matrixtype: int = 1
    # geometric description used by the checks (global structured grid)
    n_el_edge: int = 0
    kappa: Optional[np.ndarray] = None   # per global element (lexicographic), or None

    @property
    def nsub(self) -> int:
        return len(self.subdomains)


def _sub_ranges_uniform(num_el_per_sub_edge: int, num_sub_per_cube_edge: int):
    """Box partition of the cube into equal subdomain cubes, subdomain index
    x fastest, as ``prepare_subdomain_data`` (poisson_on_cube.f90:764-768)."""
    boxes = []
    for kz in range(num_sub_per_cube_edge):
        for ky in range(num_sub_per_cube_edge):
            for kx in range(num_sub_per_cube_edge):
                lo = np.array([kx, ky, kz]) * num_el_per_sub_edge
                hi = lo + num_el_per_sub_edge
                boxes.append((lo, hi))
    return boxes


def box_subdomain(isub: int, lo, hi, n_el_edge: int, kappa: Optional[np.ndarray],
                  km_ref: np.ndarray) -> Subdomain:
    """Subdomain on the element box [lo, hi) of a structured n_el_edge^3 grid
    of the unit cube, numbered like the reference example (x fastest)."""
    lo = np.asarray(lo, dtype=np.int64)
    hi = np.asarray(hi, dtype=np.int64)
    ne = hi - lo                       # elements per direction
    nn = ne + 1                        # nodes per direction
    h = 1.0 / n_el_edge
    nng = n_el_edge + 1                # global nodes per edge
    nelems = int(np.prod(ne))
    nnods = int(np.prod(nn))

    # nodes, x fastest
    k, j, i = np.meshgrid(np.arange(nn[2]), np.arange(nn[1]), np.arange(nn[0]), indexing="ij")
    ig = (lo[0] + i).ravel()
    jg = (lo[1] + j).ravel()
    kg = (lo[2] + k).ravel()
    isngn = (ig + jg * nng + kg * nng * nng).astype(np.int32)
    xyz = np.empty((3, nnods))
    xyz[0] = ig * h
    xyz[1] = jg * h
    xyz[2] = kg * h
    onb = (ig == 0) | (ig == n_el_edge) | (jg == 0) | (jg == n_el_edge) | (kg == 0) | (kg == n_el_edge)
    ifix = onb.astype(np.int32)
    fixv = np.zeros(nnods)

    # elements, x fastest
    ek, ej, ei = np.meshgrid(np.arange(ne[2]), np.arange(ne[1]), np.arange(ne[0]), indexing="ij")
    ei = ei.ravel(); ej = ej.ravel(); ek = ek.ravel()
    n1 = ei + ej * nn[0] + ek * nn[0] * nn[1]
    sx, sy = 1, nn[0]
    sz = nn[0] * nn[1]
    inet_e = np.stack([n1, n1 + sx, n1 + sx + sy, n1 + sy,
                       n1 + sz, n1 + sx + sz, n1 + sx + sy + sz, n1 + sy + sz], axis=1)
    isegn = ((lo[0] + ei) + (lo[1] + ej) * n_el_edge + (lo[2] + ek) * n_el_edge * n_el_edge).astype(np.int32)

    # element matrices: upper triangle, element by element, j outer, i <= j inner
    pairs = [(i_, j_) for j_ in range(8) for i_ in range(j_ + 1)]
    pi = np.array([p[0] for p in pairs])
    pj = np.array([p[1] for p in pairs])
    idof = inet_e[:, pi]
    jdof = inet_e[:, pj]
    i_sp = np.minimum(idof, jdof).astype(np.int32).ravel()
    j_sp = np.maximum(idof, jdof).astype(np.int32).ravel()
    scale = h * (kappa[isegn] if kappa is not None else np.ones(nelems))
    a_sp = (scale[:, None] * km_ref[pi, pj][None, :]).ravel()

    rhs = np.full(nnods, h ** 3)
    rhs[onb] = 0.0
    return Subdomain(
        isub=isub, nelems=nelems, nnods=nnods, ndofs=nnods,
        inet=inet_e.astype(np.int32).ravel(), nnet=np.full(nelems, 8, dtype=np.int32),
        nndf=np.ones(nnods, dtype=np.int32), isngn=isngn, isvgvn=isngn.copy(),
        isegn=isegn, xyz=xyz, ifix=ifix, fixv=fixv, rhs=rhs, sol=np.zeros(nnods),
        i_sparse=i_sp, j_sparse=j_sp, a_sparse=a_sp)


def poisson_on_cube(num_el_per_sub_edge: int, num_sub_per_cube_edge: int,
                    kappa: Optional[np.ndarray] = None) -> Problem:
    """The reference example: -Laplace(u) = 1 on the unit cube, u = 0 on the
    boundary, Q1 hexahedra, num_sub_per_cube_edge^3 cubic subdomains."""
    n = num_el_per_sub_edge * num_sub_per_cube_edge
    km = q1_laplace_reference_matrix()
    subs = [box_subdomain(isub, lo, hi, n, kappa, km)
            for isub, (lo, hi) in enumerate(_sub_ranges_uniform(num_el_per_sub_edge, num_sub_per_cube_edge))]
    return Problem(name=f"poisson_{n}^3_{num_sub_per_cube_edge}^3subs", nelem=n ** 3,
                   nnod=(n + 1) ** 3, ndof=(n + 1) ** 3, ndim=3, meshdim=3, subdomains=subs,
                   n_el_edge=n, kappa=kappa)


def poisson_boxes(n_el_edge: int, boxes, kappa: Optional[np.ndarray] = None, name="poisson_boxes") -> Problem:
    """Poisson on the unit cube with an arbitrary box partition (list of
    (lo, hi) element ranges that tile the grid)."""
    km = q1_laplace_reference_matrix()
    subs = [box_subdomain(isub, lo, hi, n_el_edge, kappa, km) for isub, (lo, hi) in enumerate(boxes)]
    return Problem(name=name, nelem=n_el_edge ** 3, nnod=(n_el_edge + 1) ** 3, ndof=(n_el_edge + 1) ** 3,
                   ndim=3, meshdim=3, subdomains=subs, n_el_edge=n_el_edge, kappa=kappa)


def random_box_partition(n_el_edge: int, lo_side: int, hi_side: int, seed: int):
    """Tensor-product box partition with side lengths drawn uniformly in
    [lo_side, hi_side] per axis (the last box of each axis absorbs the rest)."""
    rng = np.random.default_rng(seed)
    cuts = []
    for _ in range(3):
        c = [0]
        while c[-1] < n_el_edge:
            s = int(rng.integers(lo_side, hi_side + 1))
            if n_el_edge - (c[-1] + s) < lo_side:
                s = n_el_edge - c[-1]
            c.append(min(n_el_edge, c[-1] + s))
        cuts.append(c)
    boxes = []
    for kz in range(len(cuts[2]) - 1):
        for ky in range(len(cuts[1]) - 1):
            for kx in range(len(cuts[0]) - 1):
                boxes.append((np.array([cuts[0][kx], cuts[1][ky], cuts[2][kz]]),
                              np.array([cuts[0][kx + 1], cuts[1][ky + 1], cuts[2][kz + 1]])))
    return boxes


def lognormal_kappa(n_el_edge: int, sigma: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(sigma * rng.standard_normal(n_el_edge ** 3))


def channel_kappa(n_el_edge: int, nchannels: int = 20, width: int = 2, contrast: float = 1e4,
                  sigma: float = 2.0, seed: int = 17) -> np.ndarray:
    """Per-element coefficient exp(sigma * g), g iid N(0, 1) from `seed`, with
    `nchannels` axis-aligned channels of coefficient `contrast` and a square
    cross-section of `width` elements crossing the whole cube at random
    positions (drawn from seed + 1).  Elements are numbered x fastest."""
    kappa = np.exp(sigma * np.random.default_rng(seed).standard_normal(n_el_edge ** 3))
    rng = np.random.default_rng(seed + 1)
    k3 = kappa.reshape(n_el_edge, n_el_edge, n_el_edge)  # [z, y, x]
    w = min(width, n_el_edge)
    for _ in range(nchannels):
        axis = int(rng.integers(0, 3))
        p, q = (int(v) for v in rng.integers(0, n_el_edge - w + 1, size=2))
        if axis == 0:      # along x: fixed (y, z)
            k3[q:q + w, p:p + w, :] = contrast
        elif axis == 1:    # along y: fixed (x, z)
            k3[q:q + w, :, p:p + w] = contrast
        else:              # along z: fixed (x, y)
            k3[:, q:q + w, p:p + w] = contrast
    return kappa


def random_box_counts(n_el_edge: int, counts, lo_side: int, hi_side: int, seed: int):
    """Tensor-product box partition with counts[a] boxes along axis a, side
    lengths drawn uniformly in [lo_side, hi_side] and then adjusted (within the
    bounds) to fill the grid exactly."""
    rng = np.random.default_rng(seed)
    cuts = []
    for a in range(3):
        m = counts[a]
        if not (m * lo_side <= n_el_edge <= m * hi_side):
            raise ValueError("side bounds cannot fill the grid")
        side = rng.integers(lo_side, hi_side + 1, size=m)
        while side.sum() != n_el_edge:
            i = int(rng.integers(0, m))
            if side.sum() > n_el_edge and side[i] > lo_side:
                side[i] -= 1
            elif side.sum() < n_el_edge and side[i] < hi_side:
                side[i] += 1
        cuts.append(np.concatenate([[0], np.cumsum(side)]))
    boxes = []
    for kz in range(counts[2]):
        for ky in range(counts[1]):
            for kx in range(counts[0]):
                boxes.append((np.array([cuts[0][kx], cuts[1][ky], cuts[2][kz]]),
                              np.array([cuts[0][kx + 1], cuts[1][ky + 1], cuts[2][kz + 1]])))
    return boxes


def inclusions_young(n_el_edge: int, volume_fraction: float = 0.1, rmin: float = 3.0, rmax: float = 6.0,
                     e_matrix: float = 1.0, e_incl: float = 1e3, seed: int = 5) -> np.ndarray:
    """Per-element Young's modulus: e_matrix with spherical inclusions of
    e_incl (radius uniform in [rmin, rmax] elements, centres uniform in the
    cube, drawn from `seed`) added until they hold `volume_fraction` of the
    elements (element centres inside a sphere).  Elements are numbered x fastest."""
    rng = np.random.default_rng(seed)
    n = n_el_edge
    c = (np.arange(n) + 0.5)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    inside = np.zeros((n, n, n), dtype=bool)
    while inside.mean() < volume_fraction:
        cx, cy, cz = rng.uniform(0, n, size=3)
        r = rng.uniform(rmin, rmax)
        inside |= (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= r * r
    return np.where(inside.ravel(), e_incl, e_matrix)


def uniform_boxes(n_el_edge: int, nsub_edge: int):
    """The nsub_edge^3 equal boxes of the cube (as poisson_on_cube splits it)."""
    cuts = [round(k * n_el_edge / nsub_edge) for k in range(nsub_edge + 1)]
    return [(np.array([cuts[i], cuts[j], cuts[k]]), np.array([cuts[i + 1], cuts[j + 1], cuts[k + 1]]))
            for k in range(nsub_edge) for j in range(nsub_edge) for i in range(nsub_edge)]


def global_matrix_and_rhs(prob: Problem):
    """Assembled global stiffness matrix and load vector with the Dirichlet
    rows/columns eliminated (scipy CSR), used as an independent check."""
    import scipy.sparse as sp
    rows, cols, vals = [], [], []
    f = np.zeros(prob.ndof)
    fixed = np.zeros(prob.ndof, dtype=bool)
    cnt = np.zeros(prob.ndof)
    for s in prob.subdomains:
        g = s.isvgvn
        rows.append(g[s.i_sparse]); cols.append(g[s.j_sparse]); vals.append(s.a_sparse)
        if prob.matrixtype != 0:  # upper-triangle storage of a symmetric matrix
            off = s.i_sparse != s.j_sparse
            rows.append(g[s.j_sparse[off]]); cols.append(g[s.i_sparse[off]]); vals.append(s.a_sparse[off])
        fixed[g[s.ifix != 0]] = True
        np.add.at(f, g, s.rhs)
        np.add.at(cnt, g, 1.0)
    K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(prob.ndof, prob.ndof))
    f = f / np.maximum(cnt, 1.0)   # rhs is a restriction of the global rhs (complete)
    return K, f, fixed


def cube_connectivity(n_el_edge: int) -> np.ndarray:
    """Global node numbers (= dof numbers, one dof per node) of the 8 nodes of
    every element of the n_el_edge^3 cube grid, in global element order (x
    fastest, the order of the kappa vector), node order as in box_subdomain."""
    n = n_el_edge
    nng = n + 1
    ek, ej, ei = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    n1 = (ei + ej * nng + ek * nng * nng).ravel()
    sx, sy, sz = 1, nng, nng * nng
    return np.stack([n1, n1 + sx, n1 + sx + sy, n1 + sy,
                     n1 + sz, n1 + sx + sz, n1 + sx + sy + sz, n1 + sy + sz], axis=1).astype(np.int32)


def smooth_target(n_el_edge: int, seed: int, modes: int = 8) -> np.ndarray:
    """A seeded smooth nodal field (sum of `modes` random Fourier modes) on the
    cube grid: the target u* of the differentiation example."""
    rng = np.random.default_rng(seed)
    n = n_el_edge
    t = np.arange(n + 1) / n
    z, y, x = np.meshgrid(t, t, t, indexing="ij")
    u = np.zeros_like(x)
    for _ in range(modes):
        k = rng.integers(1, 4, size=3)
        a = rng.standard_normal() * 0.01
        ph = rng.uniform(0, 2 * np.pi, size=3)
        u += a * np.sin(np.pi * k[0] * x + ph[0]) * np.sin(np.pi * k[1] * y + ph[1]) * np.sin(np.pi * k[2] * z + ph[2])
    return u.ravel()


def q1_elasticity_reference_matrix(nu: float) -> np.ndarray:
    """24 x 24 stiffness matrix of the unit Q1 hexahedron for an isotropic
    material with E = 1, 2x2x2 Gauss integration, dofs ordered node by node
    (u_x, u_y, u_z) with the node order of box_subdomain.  For an element of
    edge h and modulus E the matrix is E * h * this."""
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2 * mu
    D[3, 3] = D[4, 4] = D[5, 5] = mu
    corners = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                        [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float)
    g = 0.5 / np.sqrt(3.0)
    K = np.zeros((24, 24))
    for gx in (0.5 - g, 0.5 + g):
        for gy in (0.5 - g, 0.5 + g):
            for gz in (0.5 - g, 0.5 + g):
                dN = np.zeros((8, 3))
                for a, (cx, cy, cz) in enumerate(corners):
                    fx = gx if cx else 1 - gx
                    fy = gy if cy else 1 - gy
                    fz = gz if cz else 1 - gz
                    sx = 1 if cx else -1
                    sy = 1 if cy else -1
                    sz = 1 if cz else -1
                    dN[a] = [sx * fy * fz, sy * fx * fz, sz * fx * fy]
                Bm = np.zeros((6, 24))
                for a in range(8):
                    Bm[0, 3 * a] = dN[a, 0]
                    Bm[1, 3 * a + 1] = dN[a, 1]
                    Bm[2, 3 * a + 2] = dN[a, 2]
                    Bm[3, 3 * a] = dN[a, 1]
                    Bm[3, 3 * a + 1] = dN[a, 0]
                    Bm[4, 3 * a + 1] = dN[a, 2]
                    Bm[4, 3 * a + 2] = dN[a, 1]
                    Bm[5, 3 * a] = dN[a, 2]
                    Bm[5, 3 * a + 2] = dN[a, 0]
                K += 0.125 * Bm.T @ D @ Bm
    return K


def elasticity_box_subdomain(isub: int, lo, hi, n_el_edge: int, young: Optional[np.ndarray],
                             ke_ref: np.ndarray) -> Subdomain:
    """Linear elasticity on the element box [lo, hi) of the unit cube grid:
    3 dofs per node, clamped at x = 0, unit body force in -z (lumped)."""
    base = box_subdomain(isub, lo, hi, n_el_edge, None, q1_laplace_reference_matrix())
    h = 1.0 / n_el_edge
    nn, ne_ = base.nnods, base.nelems
    inet_e = base.inet.reshape(ne_, 8).astype(np.int64)
    edof = (3 * inet_e[:, :, None] + np.arange(3)[None, None, :]).reshape(ne_, 24)
    pairs = [(i_, j_) for j_ in range(24) for i_ in range(j_ + 1)]
    pi = np.array([p[0] for p in pairs])
    pj = np.array([p[1] for p in pairs])
    idof, jdof = edof[:, pi], edof[:, pj]
    i_sp = np.minimum(idof, jdof).astype(np.int32).ravel()
    j_sp = np.maximum(idof, jdof).astype(np.int32).ravel()
    scale = h * (young[base.isegn] if young is not None else np.ones(ne_))
    a_sp = (scale[:, None] * ke_ref[pi, pj][None, :]).ravel()
    x0 = base.xyz[0] == 0.0
    ifix = np.repeat(x0.astype(np.int32), 3)
    ndofs = 3 * nn
    # lumped unit body force in -z: every element adds -h^3/8 to the z dof of
    # its nodes; the subdomain holds the global (complete) value, so count the
    # elements around each node in the whole grid
    ig = np.rint(base.xyz[0] / h).astype(int)
    jg = np.rint(base.xyz[1] / h).astype(int)
    kg = np.rint(base.xyz[2] / h).astype(int)
    glob_cnt = np.ones(nn)
    for ax in (ig, jg, kg):
        glob_cnt *= np.where((ax == 0) | (ax == n_el_edge), 1.0, 2.0)
    rhs = np.zeros(ndofs)
    rhs[2::3] = -glob_cnt * h ** 3 / 8.0
    rhs[ifix != 0] = 0.0
    isvgvn = (3 * base.isngn[:, None].astype(np.int64) + np.arange(3)[None, :]).ravel().astype(np.int32)
    return Subdomain(
        isub=isub, nelems=ne_, nnods=nn, ndofs=ndofs, inet=base.inet, nnet=base.nnet,
        nndf=np.full(nn, 3, dtype=np.int32), isngn=base.isngn, isvgvn=isvgvn, isegn=base.isegn,
        xyz=base.xyz, ifix=ifix, fixv=np.zeros(ndofs), rhs=rhs, sol=np.zeros(ndofs),
        i_sparse=i_sp, j_sparse=j_sp, a_sparse=a_sp)


def elasticity_on_cube(num_el_per_sub_edge: int, num_sub_per_cube_edge: int, nu: float = 0.3,
                       young: Optional[np.ndarray] = None) -> Problem:
    """Q1 linear elasticity on the unit cube: clamped at x = 0, unit body force
    in -z, cubic subdomains (the elasticity configuration at two levels)."""
    n = num_el_per_sub_edge * num_sub_per_cube_edge
    ke = q1_elasticity_reference_matrix(nu)
    subs = [elasticity_box_subdomain(isub, lo, hi, n, young, ke)
            for isub, (lo, hi) in enumerate(_sub_ranges_uniform(num_el_per_sub_edge, num_sub_per_cube_edge))]
    nnod = (n + 1) ** 3
    return Problem(name=f"elasticity_{n}^3_{num_sub_per_cube_edge}^3subs", nelem=n ** 3, nnod=nnod,
                   ndof=3 * nnod, ndim=3, meshdim=3, subdomains=subs, n_el_edge=n, kappa=young)


def body_force_loads(prob: Problem, nrhs: int, seed: int = 5) -> list:
    """nrhs load cases of an elasticity problem on the unit-cube grid: the lumped
    body force in -z of every element (-h^3/8 per node) scaled by its own iid
    N(0, 1) factor in each case.  Returns, per subdomain, an (nrhs, ndofs)
    array of complete right-hand sides (global values at the subdomain dofs,
    zero at fixed dofs)."""
    n = prob.n_el_edge
    h = 1.0 / n
    nng = n + 1
    rng = np.random.default_rng(seed)
    out = [np.zeros((nrhs, s.ndofs)) for s in prob.subdomains]
    for k in range(nrhs):
        sc = rng.standard_normal(n ** 3).reshape(n, n, n)  # [z, y, x] = global element order
        f = np.zeros((nng, nng, nng))
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    f[dz:dz + n, dy:dy + n, dx:dx + n] += sc
        f = (-h ** 3 / 8.0) * f.ravel()
        for s, o in zip(prob.subdomains, out):
            r = o[k]
            r[2::3] = f[s.isngn]
            r[s.ifix != 0] = 0.0
    return out


def q1_convection_reference_matrix(b) -> np.ndarray:
    """Galerkin convection matrix C[i][j] = int phi_i (b . grad phi_j) of the Q1
    element [0,1]^3 (node order of q1_laplace_reference_matrix).  The trilinear
    basis is a product of 1D hats, so every entry is a product of the 1D mass
    matrix [[2,1],[1,2]]/6 and the 1D convection matrix [[-1,1],[-1,1]]/2 (rows:
    test function, columns: derivative of the trial function); on an element
    of size h the matrix scales with h^2."""
    m1 = np.array([[2.0, 1.0], [1.0, 2.0]]) / 6.0
    d1 = np.array([[-0.5, 0.5], [-0.5, 0.5]])
    c = np.zeros((8, 8))
    for i in range(8):
        for j in range(8):
            oi, oj = _NODE_OFFSETS[i], _NODE_OFFSETS[j]
            f = [m1[oi[a], oj[a]] for a in range(3)]
            g = [d1[oi[a], oj[a]] for a in range(3)]
            c[i, j] = b[0] * g[0] * f[1] * f[2] + b[1] * f[0] * g[1] * f[2] + b[2] * f[0] * f[1] * g[2]
    return c


def convection_diffusion_on_cube(num_el_per_sub_edge: int, num_sub_per_cube_edge: int,
                                 b=(10.0, 7.0, 4.0)) -> Problem:
    """-Laplace(u) + b . grad(u) = 1 on the unit cube, u = 0 on the boundary,
    Q1 hexahedra, cubic subdomains: a nonsymmetric problem (matrixtype 0).
    Element matrices h K_laplace + h^2 C(b) are given in full (all 64 pairs),
    as the reference expects for general matrices."""
    n = num_el_per_sub_edge * num_sub_per_cube_edge
    h = 1.0 / n
    km = h * q1_laplace_reference_matrix() + h * h * q1_convection_reference_matrix(b)
    subs = []
    for isub, (lo, hi) in enumerate(_sub_ranges_uniform(num_el_per_sub_edge, num_sub_per_cube_edge)):
        sd = box_subdomain(isub, lo, hi, n, None, q1_laplace_reference_matrix())
        inet_e = sd.inet.reshape(sd.nelems, 8)
        ii, jj = np.meshgrid(np.arange(8), np.arange(8), indexing="ij")
        sd.i_sparse = inet_e[:, ii.ravel()].astype(np.int32).ravel()
        sd.j_sparse = inet_e[:, jj.ravel()].astype(np.int32).ravel()
        sd.a_sparse = np.tile(km[ii.ravel(), jj.ravel()], sd.nelems)
        subs.append(sd)
    return Problem(name=f"convection_diffusion_{n}^3_{num_sub_per_cube_edge}^3subs", nelem=n ** 3,
                   nnod=(n + 1) ** 3, ndof=(n + 1) ** 3, ndim=3, meshdim=3, subdomains=subs,
                   matrixtype=0, n_el_edge=n)
