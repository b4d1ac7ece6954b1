"""CPU oracle of the NeuralCE receptive-field update -- TEST INFRASTRUCTURE ONLY.

Only tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may use this module; it checks the product path and is never part of it.
numpy, float64 by default.  Restates, on the geometry of ``neuralce_gb300.nce_geometry.build_geometry``:

  h0_full        neuralce/nce/gpu_layer0_implicit.py:151-171
  delta_h0       neuralce/nce/gpu_layer0_implicit.py:189-202
  _layer_raw     neuralce/nce/local_update_implicit.py:43-54   (masked shell mean, W_self/W_shell, tanh, sigmoid gate)
  full_cache     neuralce/nce/local_update_implicit.py:89-108  ('h0' cache mode)
  energy_of      neuralce/nce/local_update_implicit.py:110-112
  local_delta    neuralce/nce/local_update_implicit.py:117-160 (slot maps == overwrite-patched copies: every duplicate
                 row of a patch carries the value of its first occurrence)
  commit         neuralce/nce/local_update_implicit.py:185-194
  accept rule    neuralce/nce/mcmc.py:178-179  (dE_eV <= 0 or u < exp(-beta dE_eV), dE_eV = dE * ys * N)

Two network variants share the code: the reference's (tanh, optional sigmoid gate, site-mean readout) and the
benchmark's (SiLU, no gate, sum readout).
"""
from __future__ import annotations

import numpy as np


def silu(x):
    return x / (1.0 + np.exp(-x))


class NCEOracle:
    def __init__(self, geo, params, mu=None, sd=None, act="tanh", pool="mean", dtype=np.float64):
        self.g = geo
        self.dt = dtype
        K1 = geo["K"] + 1
        self.mu = np.zeros(K1) if mu is None else np.asarray(mu, np.float64)
        self.sd = np.ones(K1) if sd is None else np.asarray(sd, np.float64)
        c = lambda x: np.asarray(x, dtype)
        self.P = dict(lin=c(params["lin"]), head=dict(w=c(params["head"]["w"]), b=float(params["head"]["b"])),
                      layers=[{k: c(v) for k, v in L.items()} for L in params["layers"]])
        self.act = act
        self.pool = pool
        self.norm = float(geo["nA"]) if pool == "mean" else 1.0
        N = geo["N"]
        self.active = geo["Mb"][np.arange(N) % geo["nB"]] > 1

    # ── geometry helpers ──
    def k_of(self, i):
        g = self.g; d = g["d"]; i = np.asarray(i, np.int64); c = i // g["nB"]
        return i % g["nB"], np.stack([c // (d[1] * d[2]), (c // d[2]) % d[1], c % d[2]], axis=-1)

    def site_of(self, b, k):
        d = self.g["d"]
        return ((k[..., 0] * d[1] + k[..., 1]) * d[2] + k[..., 2]) * self.g["nB"] + b

    def ball_sites(self, l, i):
        g = self.g; b, k = self.k_of(i)
        w = len(g["ball_b"][l][b])
        return self.site_of(g["ball_b"][l][b], (k[None, :] + g["ball_uo"][l][b]) % g["d"])

    def shells_of(self, sites):
        g = self.g; b, k = self.k_of(sites)
        si = self.site_of(g["Sh_b"][b], (k[:, None, None, :] + g["Sh_uo"][b]) % g["d"])     # (B, P, W)
        return np.transpose(si, (1, 0, 2)), np.transpose(g["Sh_m"][b], (1, 0, 2)).astype(np.float64)

    # ── layer 0 ──
    def h0_full(self, sig):
        g = self.g; sig = np.asarray(sig, np.int64); N, nA, K = g["N"], g["nA"], g["K"]; d = g["d"]
        c = np.arange(g["n_cells"])
        k = np.stack([c // (d[1] * d[2]), (c // d[2]) % d[1], c % d[2]], axis=-1)
        h = np.zeros((N, K))
        Mrow = g["Mb"][g["T_b"]]
        for r in range(g["Rt"]):
            sites = self.site_of(g["T_b"][r][None], (k[:, None, :] + g["T_uo"][r][None]) % d)      # (C, mo)
            th = g["theta"][Mrow[r][None], g["T_p"][r][None], sig[sites]]
            th = np.where(g["T_m"][r][None], th, 1.0)
            pr = np.prod(th, axis=-1) / g["T_ord"][r] / g["norm"][g["T_col"][r]] * nA
            for m in range(sites.shape[1]):
                if g["T_m"][r, m]:
                    np.add.at(h[:, g["T_col"][r]], sites[:, m], pr)
        return np.concatenate([self.active[:, None].astype(np.float64), h], axis=1)

    def delta_h0(self, sig, i, s_new, ov=()):
        """rows of site i: (member sites (J, mo), mask (J, mo), channel (J,), value per row (J,))"""
        g = self.g; sig = np.asarray(sig, np.int64)
        b, k = self.k_of(i)
        sites = self.site_of(g["Rv_b"][b], (k[None, None, :] + g["Rv_uo"][b]) % g["d"])
        Mv = g["Mb"][g["Rv_b"][b]]

        def prod(ovx):
            sp = sig[sites].copy()
            for (ss, v) in ovx:
                sp = np.where(sites == ss, v, sp)
            th = np.where(g["Rv_m"][b], g["theta"][Mv, g["Rv_p"][b], sp], 1.0)
            return np.prod(th, axis=-1)
        dpi = prod(tuple(ov) + ((i, s_new),)) - prod(ov)
        w = np.where(g["Rv_v"][b], dpi / g["Rv_ord"][b] / g["norm"][g["Rv_col"][b]] * g["nA"], 0.0)
        ok = g["Rv_m"][b] & g["Rv_v"][b][:, None]
        return sites, ok, g["Rv_col"][b] + 1, w

    # ── layers ──
    def _activation(self, pre):
        return np.tanh(pre) if self.act == "tanh" else silu(pre)

    def layer(self, L, h_prev, sites):
        si, sm = self.shells_of(sites)
        m = sm[..., None]
        gth = h_prev[si]
        z = (gth * m).sum(-2) / np.maximum(sm.sum(-1), 1.0)[..., None]                   # (P, B, C)
        pre = h_prev[sites] @ L["self"] + np.einsum("pbc,pcd->bd", z, L["shell"]) + L["b"]
        out = self._activation(pre)
        if "gate" in L:
            gz = np.einsum("pbc,pcd->bd", z, L["gate"]) + L["gb"]
            out = out * (1.0 / (1.0 + np.exp(-gz)))
        return out

    def h0s(self, sig):
        h = self.h0_full(sig)
        return np.where(self.active[:, None], (h - self.mu) / self.sd, 0.0).astype(self.dt)

    def full_cache(self, sig):
        h0 = self.h0s(sig)
        hs = [h0]
        allsites = np.arange(self.g["N"])
        for L in self.P["layers"]:
            hs.append(self.layer(L, hs[-1], allsites))
        e = h0 @ self.P["lin"]
        if self.P["layers"]:
            e = e + hs[-1] @ self.P["head"]["w"]
        e = np.where(self.active, e, 0.0)
        return dict(h0=h0, hmid=hs[1:-1], hL=hs[-1], e=e)

    def energy_of(self, cache):
        return float(cache["e"].sum() / self.norm + self.P["head"]["b"])

    def energy(self, sig):
        return self.energy_of(self.full_cache(sig))

    # ── local update ──
    def local_delta(self, cache, sig, flips):
        """flips: [(site, new species), ...] applied in order.  Returns (dE, patch)."""
        Kc = self.g["K"] + 1
        b0 = np.concatenate([self.ball_sites(0, f[0]) for f in flips])
        first0 = {}
        for q, s in enumerate(b0):
            first0.setdefault(int(s), q)
        acc = np.zeros((len(b0), Kc))
        ov = []
        for (i, s_new) in flips:
            sites, ok, chan, w = self.delta_h0(sig, i, s_new, ov)
            for j in range(sites.shape[0]):
                for m in range(sites.shape[1]):
                    if ok[j, m]:
                        q = first0.get(int(sites[j, m]))
                        if q is not None:
                            acc[q, chan[j]] += w[j] / self.sd[chan[j]]
            ov.append((i, s_new))
        acc = acc[[first0[int(s)] for s in b0]]
        h0_new = cache["h0"][b0] + acc
        h0p = cache["h0"].copy(); h0p[b0] = h0_new
        patch = dict(h0=(b0, h0_new), hmid=[])
        nL = len(self.P["layers"])
        if nL == 0:
            rows, e_new = b0, h0_new @ self.P["lin"]
        else:
            prev = h0p
            for l, L in enumerate(self.P["layers"]):
                bl = np.concatenate([self.ball_sites(l + 1, f[0]) for f in flips])
                v = self.layer(L, prev, bl)
                if l + 1 < nL:
                    patch["hmid"].append((bl, v))
                    prev = cache["hmid"][l].copy(); prev[bl] = v
                rows, vals = bl, v
            e_new = h0p[rows] @ self.P["lin"] + vals @ self.P["head"]["w"]
            patch["hL"] = (rows, vals)
        e_new = np.where(self.active[rows], e_new, 0.0)
        seen = set(); dE = 0.0
        for q, s in enumerate(rows):
            if int(s) not in seen:
                seen.add(int(s)); dE += e_new[q] - cache["e"][s]
        patch["e"] = (rows, e_new)
        return dE / self.norm, patch

    def commit(self, cache, patch, accept):
        if not accept:
            return cache
        out = dict(cache)
        for k in ("h0", "e", "hL"):
            if k in patch:
                r, v = patch[k]; a = cache[k].copy(); a[r] = v; out[k] = a
        out["hmid"] = []
        for l, (r, v) in enumerate(patch["hmid"]):
            a = cache["hmid"][l].copy(); a[r] = v; out["hmid"].append(a)
        return out


def expand_params(mdl, seed_idx=0):
    """model.pkl parameters on the full layer-0 channel list (``neuralce/nce/mc_model.py:36-57``): zero rows for the
    channels the model dropped, mu = 0 / sd = 1 there."""
    keep = np.asarray(mdl["keep"]); Kfull = int(mdl["K_chem"])
    P = mdl["params"][seed_idx]
    lin = np.zeros(Kfull); lin[keep] = P["lin"]
    layers = []
    for L in P["layers"]:
        if L["self"].shape[0] == len(keep):
            Lx = dict(L)
            Lx["self"] = np.zeros((Kfull, L["self"].shape[1])); Lx["self"][keep] = L["self"]
            Lx["shell"] = np.zeros((L["shell"].shape[0], Kfull, L["shell"].shape[2])); Lx["shell"][:, keep] = L["shell"]
            if "gate" in L:
                Lx["gate"] = np.zeros((L["gate"].shape[0], Kfull, L["gate"].shape[2])); Lx["gate"][:, keep] = L["gate"]
            if "shell_max" in L:
                raise NotImplementedError("shell_max layers")
            layers.append(Lx)
        else:
            layers.append(dict(L))
    mu = np.zeros(Kfull); sd = np.ones(Kfull); mu[keep] = mdl["mu"]; sd[keep] = mdl["sd"]
    return dict(lin=lin, layers=layers, head=dict(P["head"])), mu, sd


def run_chain(orc, cache, sig, prop_i, prop_j, u, beta, scale_eV):
    """Metropolis chain of one replica on a host proposal stream (``neuralce/nce/mcmc.py:167-185``): flips
    [[i, sig[j]], [j, sig[i]]]; same species is an accepted no-op; accept if dE_eV <= 0 or u < exp(-beta dE_eV).
    Returns (cache, sig, E change, accepted count, dE per step, min Metropolis margin)."""
    sig = np.asarray(sig, np.int64).copy()
    dEs, nacc, dsum, margin = [], 0, 0.0, np.inf
    for i, j, uu in zip(prop_i, prop_j, u):
        i, j = int(i), int(j)
        if sig[i] == sig[j]:
            dEs.append(0.0); nacc += 1; continue
        dE, patch = orc.local_delta(cache, sig, [(i, int(sig[j])), (j, int(sig[i]))])
        dEeV = dE * scale_eV
        acc = dEeV <= 0 or uu < np.exp(-beta * dEeV)
        if dEeV > 0:
            margin = min(margin, abs(np.log(uu) + beta * dEeV))
        dEs.append(dE)
        if acc:
            cache = orc.commit(cache, patch, True)
            sig[i], sig[j] = sig[j], sig[i]
            nacc += 1; dsum += dE
    return cache, sig, dsum, nacc, np.array(dEs), margin


def trace_chain(orc, cache, sig, prop_i, prop_j, u, beta, scale_eV, dE_engine, near_eV):
    """Step-by-step check of an engine's Metropolis chain of one replica against this oracle.

    The engine reports its dE of every step (``dE_engine``, model units; 0 for same-species draws).  Its decision
    at a step is the reference rule (``neuralce/nce/mcmc.py:178-179``) applied to its own dE.  At each step the
    oracle evaluates the same swap with its float64 dE and decides by the same rule.  Where the two decisions
    differ, the step must be near its threshold -- the oracle's margin |dE_eV + ln(u) / beta| below ``near_eV`` --
    or it is reported as a mismatch; either way the oracle then follows the engine's decision, so that every later
    step is still checked.  Returns a dict: sig and cache after the followed chain, per-step oracle dE, the steps
    whose decisions differ (``excused`` near the threshold, ``mismatch`` elsewhere), the number of steps the
    engine's dE puts near the threshold (``near_engine``: what the engine counts) and the accepted count."""
    sig = np.asarray(sig, np.int64).copy()
    out = dict(dE=[], excused=[], mismatch=[], near_engine=0, nacc=0)
    for k, (i, j, uu) in enumerate(zip(prop_i, prop_j, u)):
        i, j = int(i), int(j)
        if sig[i] == sig[j]:
            out["dE"].append(0.0); out["nacc"] += 1
            continue
        dE, patch = orc.local_delta(cache, sig, [(i, int(sig[j])), (j, int(sig[i]))])
        out["dE"].append(dE)
        de_o, de_e = dE * scale_eV, float(dE_engine[k]) * scale_eV
        acc_o = de_o <= 0 or uu < np.exp(-beta * de_o)
        acc_e = de_e <= 0 or uu < np.exp(-beta * de_e)
        if beta > 0 and abs(de_e + np.log(uu) / beta) < near_eV:
            out["near_engine"] += 1
        if acc_o != acc_e:
            near_o = beta > 0 and abs(de_o + np.log(uu) / beta) < near_eV
            out["excused" if near_o else "mismatch"].append(k)
        if acc_e:
            cache = orc.commit(cache, patch, True)
            sig[i], sig[j] = sig[j], sig[i]
            out["nacc"] += 1
    out["sig"], out["cache"], out["dE"] = sig, cache, np.array(out["dE"])
    return out
