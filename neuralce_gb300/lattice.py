"""Integer lattice algebra and cluster-orbit enumeration for the implicit (template-only) tables.

Everything here runs once at setup on the host.  It replaces the pieces of the reference's setup that
came from sympy and icet, which are not available to this package:

* ``smith_normal_form``  -- own elimination algorithm (the reference calls sympy's
  ``smith_normal_decomp``, ``neuralce/ce/ce_gpu_implicit.py:28-39``).  The diagonal ``d`` is the unique
  invariant-factor form; ``U`` may differ from sympy's, which only changes the internal canonical site
  order (``perm`` / ``inv_perm`` map it back to the input order, as in the reference).
* ``site_decompose`` / ``canonical_cells`` -- same contract as ``neuralce/nce/gpu_layer0_tiled.py:16-33`` and
  ``neuralce/ce/ce_gpu_implicit.py:42-46``.
* ``space_group`` + ``enumerate_orbits`` -- the primitive orbit list that icet 3.2 (``ClusterSpace``,
  ``cs._orbit_list``) provides to ``build_ce_gpu_implicit`` (``ce_gpu_implicit.py:56-86``) and to
  ``build_template`` (``neuralce/nce/gpu_layer0_tiled.py:36-53``).  Clusters of order k contain only active
  sites (more than one allowed species), every pair distance is within ``cutoffs[k-2]`` (icet's
  "longest distance between two sites" rule), orbits are the space-group classes of clusters, and the
  orbit list is sorted by (order, radius, sorted pair distances) with radius = mean distance of the sites
  to their geometric centre (icet's ``Cluster.radius``).  Orbits with equal (order, radius, distances)
  are ordered by a deterministic key of the canonical representative.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

# ───────────────────────────── Smith normal form (3x3 integer) ─────────────────────────────────

def smith_normal_form(T):
    """U, d, V with U @ T @ V = diag(d), U, V unimodular, d > 0 and d[0] | d[1] | d[2]."""
    A = np.array(T, dtype=object)
    n = A.shape[0]
    U = np.eye(n, dtype=object)
    V = np.eye(n, dtype=object)
    for t in range(n):
        while True:
            # pivot: smallest non-zero |entry| in the trailing block
            best = None
            for i in range(t, n):
                for j in range(t, n):
                    if A[i, j] != 0 and (best is None or abs(A[i, j]) < abs(A[best])):
                        best = (i, j)
            if best is None:
                break
            i, j = best
            A[[t, i]] = A[[i, t]]; U[[t, i]] = U[[i, t]]
            A[:, [t, j]] = A[:, [j, t]]; V[:, [t, j]] = V[:, [j, t]]
            done = True
            p = A[t, t]
            for i in range(t + 1, n):                      # clear column t
                q = A[i, t] // p
                if q:
                    A[i] = A[i] - q * A[t]; U[i] = U[i] - q * U[t]
                if A[i, t] != 0:
                    done = False
            for j in range(t + 1, n):                      # clear row t
                q = A[t, j] // p
                if q:
                    A[:, j] = A[:, j] - q * A[:, t]; V[:, j] = V[:, j] - q * V[:, t]
                if A[t, j] != 0:
                    done = False
            if not done:
                continue
            # divisibility: p must divide every entry of the trailing block
            bad = None
            for i in range(t + 1, n):
                for j in range(t + 1, n):
                    if A[i, j] % p != 0:
                        bad = i
                        break
                if bad is not None:
                    break
            if bad is None:
                break
            A[t] = A[t] + A[bad]; U[t] = U[t] + U[bad]      # bring the offending row up and repeat
        if A[t, t] < 0:
            A[t] = -A[t]; U[t] = -U[t]
    d = np.array([int(A[i, i]) for i in range(n)], np.int64)
    U = np.array(U, dtype=np.int64); V = np.array(V, dtype=np.int64)
    assert np.array_equal(U @ np.asarray(T, np.int64) @ V, np.diag(d)), "SNF does not reproduce T"
    assert (d > 0).all(), f"singular supercell matrix {T}"
    assert abs(round(np.linalg.det(U.astype(float)))) == 1 and abs(round(np.linalg.det(V.astype(float)))) == 1
    return U, d, V


def canonical_cells(off, U, d):
    """Integer primitive-cell offsets (...,3) -> SNF coordinate k = U n mod d and the cell index
    (k0*d1 + k1)*d2 + k2 (``neuralce/ce/ce_gpu_implicit.py:42-46``)."""
    k = np.mod(np.asarray(off, np.int64) @ U.T, d)
    return k, (k[..., 0] * d[1] + k[..., 1]) * d[2] + k[..., 2]


def site_decompose(prim_cell, prim_frac, cell, positions, tol=1e-3):
    """Every supercell site -> (basis index, integer primitive-cell offset reduced into the supercell),
    integer supercell matrix T (rows of ``cell`` = T @ prim_cell) and the number of primitive cells
    (``neuralce/nce/gpu_layer0_tiled.py:16-33``)."""
    P = np.asarray(prim_cell, float); S = np.asarray(cell, float)
    T = S @ np.linalg.inv(P)
    if not np.allclose(T, np.round(T), atol=1e-4):
        raise ValueError(f"supercell is not an integer multiple of the primitive: T={T}")
    T = np.round(T).astype(np.int64)
    n_cells = int(round(abs(np.linalg.det(T))))
    F = np.asarray(positions, float) @ np.linalg.inv(P)
    pb = np.asarray(prim_frac, float)
    n = len(F)
    basis = np.full(n, -1, np.int64); off = np.zeros((n, 3), np.int64); best = np.full(n, np.inf)
    for b in range(len(pb)):
        dlt = F - pb[b]; t = np.round(dlt); err = np.abs(dlt - t).max(1)
        take = err < best
        basis[take] = b; off[take] = t[take]; best[take] = err[take]
    if n and best.max() >= tol:
        raise ValueError(f"site does not sit on the primitive lattice (max err {best.max():.2e})")
    Tinv = np.linalg.inv(T)
    off_red = off - np.floor(off @ Tinv + 1e-9).astype(np.int64) @ T
    return basis, off_red, T, n_cells


# ───────────────────────────── primitive structure + symmetry ──────────────────────────────────

@dataclass
class Primitive:
    """Primitive structure of a cluster space: lattice rows ``cell`` (A), fractional basis positions, the
    allowed species per basis site (icet order: sorted by atomic number)."""
    cell: np.ndarray
    frac: np.ndarray
    species: list
    numbers: np.ndarray = None

    @property
    def nB(self):
        return len(self.frac)

    def cart(self, b, n):
        return (np.asarray(self.frac)[b] + np.asarray(n, float)) @ np.asarray(self.cell, float)


def space_group(prim: Primitive, tol=1e-5):
    """Space-group operations (W, t) in fractional coordinates, x' = W x + t, that map every basis site
    onto a basis site with the same allowed species.  W is an integer matrix acting on fractional
    coordinates (columns are the images of the lattice vectors' reciprocal coordinates)."""
    A = np.asarray(prim.cell, float)
    G = A @ A.T
    lengths = np.sqrt(np.diag(G))
    rng = range(-2, 3)
    cands = [[] for _ in range(3)]
    for n in itertools.product(rng, rng, rng):
        v = np.asarray(n, float) @ A
        L = np.linalg.norm(v)
        for i in range(3):
            if abs(L - lengths[i]) < tol * max(1.0, lengths[i]):
                cands[i].append(np.asarray(n, np.int64))
    ops = []
    frac = np.mod(np.asarray(prim.frac, float), 1.0)
    key = [tuple(sorted(s)) for s in prim.species]
    for r0 in cands[0]:
        for r1 in cands[1]:
            for r2 in cands[2]:
                M = np.stack([r0, r1, r2])                     # row i = image of lattice vector i (integer coords)
                if abs(round(np.linalg.det(M.astype(float)))) != 1:
                    continue
                if not np.allclose(M @ G @ M.T, G, atol=tol * max(1.0, G.max())):
                    continue
                W = M.T                                          # fractional coords transform: x' = W x
                x0 = W @ frac[0]
                for j in range(len(frac)):
                    if key[j] != key[0]:
                        continue
                    t = np.mod(frac[j] - x0, 1.0)
                    ok = True
                    for b in range(len(frac)):
                        y = np.mod(W @ frac[b] + t, 1.0)
                        dd = np.abs(((frac - y) + 0.5) % 1.0 - 0.5).max(1)
                        m = np.where(dd < 1e-4)[0]
                        if len(m) != 1 or key[m[0]] != key[b]:
                            ok = False
                            break
                    if ok:
                        ops.append((W.astype(np.int64), t))
    return ops


def _apply_op(op, prim_frac, b, n):
    """image of lattice site (b, n) under op -> (b', n')"""
    W, t = op
    x = W @ (np.asarray(prim_frac[b], float) + np.asarray(n, float)) + t
    frac = np.asarray(prim_frac, float)
    for bb in range(len(frac)):
        dlt = x - frac[bb]
        r = np.round(dlt)
        if np.abs(dlt - r).max() < 1e-4:
            return bb, tuple(int(v) for v in r)
    raise AssertionError("symmetry operation maps a site off the lattice")


def _canon(cluster):
    """translation-canonical form of a cluster (tuple of (b, (n0,n1,n2))): the lexicographically smallest
    sorted tuple over all choices of the member translated to offset 0."""
    best = None
    for (_, n0) in cluster:
        c = tuple(sorted((b, (n[0] - n0[0], n[1] - n0[1], n[2] - n0[2])) for (b, n) in cluster))
        if best is None or c < best:
            best = c
    return best


@dataclass
class Orbit:
    order: int
    radius: float
    distances: tuple
    clusters: list = field(default_factory=list)   # translation classes: list of tuples of (b, (n0,n1,n2))

    @property
    def representative(self):
        return self.clusters[0]


def _geometry(prim, cluster):
    pts = np.array([prim.cart(b, n) for (b, n) in cluster])
    ctr = pts.mean(0)
    radius = float(np.linalg.norm(pts - ctr, axis=1).mean())
    dist = tuple(sorted(round(float(np.linalg.norm(pts[i] - pts[j])), 6)
                        for i in range(len(pts)) for j in range(i + 1, len(pts))))
    return radius, dist


def enumerate_orbits(prim: Primitive, cutoffs, tol=1e-5):
    """Orbit list of the primitive: singlets of every active basis site, then clusters of order
    2..len(cutoffs)+1 with all pair distances <= cutoffs[order-2].  Returns a list of Orbit sorted by
    (order, radius, distances, canonical representative)."""
    active = [b for b in range(prim.nB) if len(prim.species[b]) > 1]
    ops = space_group(prim, tol)
    rmax = max(cutoffs) if len(cutoffs) else 0.0
    # neighbours of each active basis site within the largest cutoff
    A = np.asarray(prim.cell, float)
    span = int(math.ceil(rmax / min(np.linalg.norm(np.cross(A[1], A[2])), np.linalg.norm(np.cross(A[2], A[0])),
                                    np.linalg.norm(np.cross(A[0], A[1]))) * np.abs(np.linalg.det(A)))) + 1 if rmax > 0 else 0
    nbr = {}
    for b in active:
        lst = []
        r0 = prim.cart(b, (0, 0, 0))
        for n in itertools.product(range(-span, span + 1), repeat=3):
            for bb in active:
                if bb == b and n == (0, 0, 0):
                    continue
                dist = np.linalg.norm(prim.cart(bb, n) - r0)
                if dist <= rmax + tol:
                    lst.append(((bb, n), dist))
        nbr[b] = lst
    classes = {}
    for b in active:                                       # singlets
        classes[_canon(((b, (0, 0, 0)),))] = 1
    for order in range(2, len(cutoffs) + 2):
        cut = cutoffs[order - 2]
        for b in active:
            anchor = (b, (0, 0, 0))
            cand = [s for (s, dist) in nbr[b] if dist <= cut + tol]
            pos = {s: prim.cart(s[0], s[1]) for s in cand}
            for combo in itertools.combinations(cand, order - 1):
                ok = True
                for i in range(len(combo)):
                    for j in range(i + 1, len(combo)):
                        if np.linalg.norm(pos[combo[i]] - pos[combo[j]]) > cut + tol:
                            ok = False
                            break
                    if not ok:
                        break
                if ok:
                    classes[_canon((anchor,) + combo)] = order
    seen = set()
    orbits = []
    for c in sorted(classes):
        if c in seen:
            continue
        members = set()
        for op in ops:
            img = tuple(_apply_op(op, prim.frac, b, n) for (b, n) in c)
            members.add(_canon(img))
        seen |= members
        radius, dist = _geometry(prim, c)
        o = Orbit(order=len(c), radius=radius, distances=dist, clusters=sorted(members))
        orbits.append(o)
    orbits.sort(key=lambda o: (o.order, round(o.radius, 5), o.distances, o.representative))
    return orbits


# ───────────────────────────── point functions ─────────────────────────────────────────────────

def theta(M, p, s):
    """Orthonormal point function of icet for M species (``neuralce/nce/gpu_layer0.py:32-35``)."""
    k = (p + 2) // 2
    x = 2.0 * np.pi * k * s / M
    return -np.cos(x) if p % 2 == 0 else -np.sin(x)
