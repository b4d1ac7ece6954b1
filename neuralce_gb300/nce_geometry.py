"""Template-only geometry of the NeuralCE receptive-field update (host setup).

Restates ``build_geometry`` (``neuralce/nce/gpu_layer0_implicit.py:17-118``) and ``build_template``
(``neuralce/nce/gpu_layer0_tiled.py:36-53``) from the orbit list of ``lattice.enumerate_orbits``:

* layer-0 template rows (basis, offset, point-function index, column, order; count per column) and the
  reverse rows per basis site (every (row, slot) whose member has that basis, relative to the slot);
* ``h0`` columns: channel 0 = active-site indicator, channel 1 + col = nA * sum over the instances containing
  the site of prod(theta) / (order * count_col * n_cells) (site mean = the cluster vector);
* shells: partners per basis site and shell (``shell_edges`` bins, active-active, periodic images kept);
* balls: ball0 = member offsets of the reverse rows, ball_{l+1} = ball_l grown by the partner offsets.

Offsets are kept in primitive-lattice coordinates; ``uo(off) = U off mod d`` converts them for a supercell.
"""
from __future__ import annotations

import itertools
import math

import numpy as np

from .io import Z_OF
from .lattice import canonical_cells, site_decompose, smith_normal_form, theta


def build_template(cs):
    """NCE template rows of the primitive orbit list (binary: one cluster-vector element per orbit)."""
    tb, to, tp, tcol, tord, cnt = [], [], [], [], [], []
    for col, o in enumerate(cs.orbits):
        n = 0
        for inst in o.clusters:
            tb.append([s[0] for s in inst]); to.append([s[1] for s in inst]); tp.append([0] * len(inst))
            tcol.append(col); tord.append(len(inst)); n += 1
        cnt.append(n)
    mo = max(len(r) for r in tb); Rt = len(tb)
    B = np.zeros((Rt, mo), np.int64); O = np.zeros((Rt, mo, 3), np.int64)
    Pp = np.zeros((Rt, mo), np.int32); M = np.zeros((Rt, mo), bool)
    for r in range(Rt):
        k = len(tb[r]); B[r, :k] = tb[r]; O[r, :k] = to[r]; Pp[r, :k] = tp[r]; M[r, :k] = True
    return dict(basis=B, off=O, pidx=Pp, mask=M, col=np.asarray(tcol, np.int32), order=np.asarray(tord, np.int32),
                count=np.asarray(cnt, float), K=len(cs.orbits), mo=mo)


def _partners(prim, active_b, shell_edges):
    """per basis site, per shell: (basis, offset) of active partners within the shell (distance bins (lo, hi])."""
    edges = np.asarray(shell_edges, float)
    rmax = float(edges[-1]) + 1e-6
    A = np.asarray(prim.cell, float)
    vol = abs(np.linalg.det(A))
    hmin = min(vol / np.linalg.norm(np.cross(A[(i + 1) % 3], A[(i + 2) % 3])) for i in range(3))
    span = int(math.ceil(rmax / hmin)) + 1
    P = len(edges) - 1
    part = [[[] for _ in range(P)] for _ in range(prim.nB)]
    for b in range(prim.nB):
        if b not in active_b:
            continue
        r0 = prim.cart(b, (0, 0, 0))
        for n in itertools.product(range(-span, span + 1), repeat=3):
            for bb in active_b:
                d = np.linalg.norm(prim.cart(bb, n) - r0)
                if 1e-6 < d <= rmax:
                    sh = int(np.digitize([d], edges[1:-1], right=True)[0])
                    part[b][sh].append((bb, tuple(int(x) for x in n)))
    return part


def build_geometry(cs, structure, shell_edges, depth):
    prim = cs.primitive; nB = prim.nB
    basis, off_red, T, n_cells = site_decompose(prim.cell, prim.frac, structure.cell, structure.positions)
    N = len(structure)
    if N != nB * n_cells:
        raise ValueError(f"{N} sites for {nB} basis sites x {n_cells} cells")
    U, d, _ = smith_normal_form(T.T)
    _, cell_idx = canonical_cells(off_red, U, d)
    canon = cell_idx * nB + basis
    if len(np.unique(canon)) != N:
        raise ValueError("sites do not form a clean tiling of the primitive")
    perm = np.argsort(canon).astype(np.int64); inv_perm = np.empty(N, np.int64); inv_perm[perm] = np.arange(N)
    uo = lambda o: np.mod(np.asarray(o, np.int64) @ U.T, d).astype(np.int32)
    Mb = np.array([len(s) for s in prim.species], np.int32)
    active_b = [int(b) for b in np.where(Mb > 1)[0]]
    nA = len(active_b) * n_cells
    # species index per site: rank of Z within the basis site's allowed species
    sig_in = np.zeros(N, np.int8)
    for b in range(nB):
        m = basis == b
        lut = {Z_OF[s]: k for k, s in enumerate(sorted(prim.species[b], key=lambda x: Z_OF[x]))}
        z = structure.numbers[m]
        bad = sorted(set(int(x) for x in np.unique(z)) - set(lut))
        if bad:
            raise ValueError(f"basis {b}: atomic numbers {bad} not in {prim.species[b]}")
        tab = np.zeros(256, np.int8)
        for zz, k in lut.items():
            tab[zz] = k
        sig_in[m] = tab[z]
    tpl = build_template(cs)
    Rt, mo = tpl["basis"].shape; K = int(tpl["K"])
    msk = tpl["mask"]; T_b = tpl["basis"].astype(np.int32).copy(); T_off = tpl["off"].copy()
    for r in range(Rt):
        for m in range(mo):
            if not msk[r, m]:
                T_b[r, m] = T_b[r, 0]; T_off[r, m] = T_off[r, 0]
    maxM = int(Mb.max()); maxP = max(int(tpl["pidx"].max()) + 1, 1)
    th = np.zeros((maxM + 1, maxP, maxM))
    for Mv in range(1, maxM + 1):
        for p in range(maxP):
            for s in range(Mv):
                th[Mv, p, s] = theta(Mv, p, s)
    ent = [[] for _ in range(nB)]
    for r in range(Rt):
        for m in range(mo):
            if msk[r, m]:
                ent[T_b[r, m]].append((r, m))
    J = max(len(e) for e in ent)
    Rv_b = np.zeros((nB, J, mo), np.int32); Rv_off = np.zeros((nB, J, mo, 3), np.int64)
    Rv_p = np.zeros((nB, J, mo), np.int32); Rv_m = np.zeros((nB, J, mo), bool)
    Rv_col = np.zeros((nB, J), np.int32); Rv_ord = np.ones((nB, J), np.float64); Rv_v = np.zeros((nB, J), bool)
    ball0 = [set() for _ in range(nB)]
    for b in range(nB):
        Rv_b[b] = b
        for j, (r, m) in enumerate(ent[b]):
            rel = T_off[r] - T_off[r, m]
            Rv_b[b, j] = T_b[r]; Rv_off[b, j] = rel; Rv_p[b, j] = tpl["pidx"][r]; Rv_m[b, j] = msk[r]
            Rv_col[b, j] = tpl["col"][r]; Rv_ord[b, j] = tpl["order"][r]; Rv_v[b, j] = True
            for mm in range(mo):
                if msk[r, mm]:
                    ball0[b].add((int(T_b[r, mm]), tuple(int(x) for x in rel[mm])))
    part = _partners(prim, active_b, shell_edges)
    P = len(shell_edges) - 1
    W = max(max(len(part[b][p]) for p in range(P)) for b in range(nB))
    Sh_b = np.zeros((nB, P, W), np.int32); Sh_off = np.zeros((nB, P, W, 3), np.int64); Sh_m = np.zeros((nB, P, W), bool)
    for b in range(nB):
        Sh_b[b] = b
        for p in range(P):
            for w, (bb, o) in enumerate(part[b][p]):
                Sh_b[b, p, w] = bb; Sh_off[b, p, w] = o; Sh_m[b, p, w] = True
    partners = [set((bb, o) for p in range(P) for (bb, o) in part[b][p]) for b in range(nB)]
    balls = [ball0]
    for _ in range(depth):
        prev = balls[-1]; nxt = []
        for b in range(nB):
            s = set(prev[b])
            for (bb, o) in prev[b]:
                for (b2, o2) in partners[bb]:
                    s.add((b2, (o[0] + o2[0], o[1] + o2[1], o[2] + o2[2])))
            nxt.append(s)
        balls.append(nxt)
    ball_b, ball_off, ball_n = [], [], []
    for bl in balls:
        w = max(len(s) for s in bl)
        Bb = np.zeros((nB, w), np.int32); Bo = np.zeros((nB, w, 3), np.int64); Bn = np.zeros(nB, np.int32)
        for b in range(nB):
            Bb[b] = b; items = sorted(bl[b]); Bn[b] = len(items)
            for q, (bb, o) in enumerate(items):
                Bb[b, q] = bb; Bo[b, q] = o
        ball_b.append(Bb); ball_off.append(Bo); ball_n.append(Bn)
    grp_sl = {}
    for b in active_b:
        grp_sl.setdefault(tuple(prim.species[b]), []).append(b)
    grp = list(grp_sl.values())
    maxb = max(len(g) for g in grp)
    grp_b = np.zeros((len(grp), maxb), np.int32); grp_nb = np.zeros(len(grp), np.int32)
    for g, bs in enumerate(grp):
        grp_b[g, :len(bs)] = bs; grp_nb[g] = len(bs)
    return dict(N=N, nB=nB, n_cells=n_cells, nA=nA, K=K, mo=mo, Rt=Rt, J=J, P=P, W=W, depth=depth, d=d.astype(np.int64),
                U=U, T=T, perm=perm, inv_perm=inv_perm, basis_in=basis, sig=sig_in[perm], Mb=Mb, active_b=active_b,
                theta=th, norm=tpl["count"] * n_cells, count=tpl["count"],
                T_b=T_b, T_off=T_off, T_uo=uo(T_off), T_p=tpl["pidx"].astype(np.int32), T_m=msk,
                T_col=tpl["col"].astype(np.int32), T_ord=tpl["order"].astype(np.float64),
                Rv_b=Rv_b, Rv_off=Rv_off, Rv_uo=uo(Rv_off), Rv_p=Rv_p, Rv_m=Rv_m, Rv_col=Rv_col, Rv_ord=Rv_ord, Rv_v=Rv_v,
                Sh_b=Sh_b, Sh_off=Sh_off, Sh_uo=uo(Sh_off), Sh_m=Sh_m,
                ball_b=ball_b, ball_off=ball_off, ball_uo=[uo(x) for x in ball_off], ball_w=[x.shape[1] for x in ball_b], ball_n=ball_n,
                grp_b=grp_b, grp_nb=grp_nb)
