"""NeuralCE on the GB300 engine: ``load_model`` / ``setup(mdl, atoms)`` and the device PT state.

Mirrors ``neuralce/nce/mc_model.py``: ``load_model`` (``:20-21``), ``expand_params`` (``:36-57``: zero rows for the
layer-0 channels the model dropped), ``setup`` / ``setup_implicit`` (``:60-111,175-228``) returning a dict with
``energy``, ``full_cache``, ``local_delta``-style stepping, ``perm`` / ``inv_perm``, ``to_eV_per_atom`` and
``dE_eV_total``.  The receptive-field update runs in libnce_gb300 (``nce_nce_run_chunk``); geometry comes from
``nce_geometry.build_geometry``.

Two network families share the engine:
  * model.pkl networks (tanh, optional sigmoid gate, site-mean readout, eV via ys/ym) -- the reference's;
  * the benchmark network (``synthetic_model``): depth 3, width 64, SiLU, sum readout, one 12-neighbour shell,
    weights ~ N(0, 1/fan_in) from a seed, energies directly in eV.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .ce_tables import ClusterSpace
from .io import Structure, load_model  # noqa: F401  (re-exported, reference name)
from .nce_geometry import build_geometry


def expand_params(mdl, seed_idx=0):
    """model.pkl parameters on the full layer-0 channel list; mu = 0 / sd = 1 on dropped channels."""
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
                raise NotImplementedError("shell_max (masked max) layers are not on this engine")
            layers.append(Lx)
        else:
            layers.append(dict(L))
    mu = np.zeros(Kfull); sd = np.ones(Kfull); mu[keep] = mdl["mu"]; sd[keep] = mdl["sd"]
    return dict(lin=lin, layers=layers, head=dict(P["head"])), mu, sd


def synthetic_model(C0, depth=3, width=64, P=1, seed=0):
    """Benchmark network: weights and biases ~ N(0, 1/fan_in) from ``seed``."""
    rng = np.random.default_rng(seed)
    g = lambda shape, fan: rng.normal(0.0, 1.0 / np.sqrt(fan), shape)
    layers = []
    cin = C0
    for _ in range(depth):
        layers.append(dict(self=g((cin, width), cin), shell=g((P, cin, width), cin), b=g((width,), cin)))
        cin = width
    return dict(lin=g((C0,), C0), layers=layers, head=dict(w=g((width,), width), b=0.0))


def tc_gemm(A, B, split=False):
    """A @ B on the tensor-core tile path of the layers (tcgen05): float32 CUDA tensors A (M, K), B (K, N) with
    M % 128 == 0, N % 16 == 0 (16..256), K <= 256; operands rounded to bf16 (``split``: hi + lo pairs)."""
    import torch
    A = A.contiguous().float(); B = B.contiguous().float()
    M, K = A.shape; N = B.shape[1]
    out = torch.empty(M, N, dtype=torch.float32, device=A.device)
    _lib.check(_lib.lib().nce_tc_gemm(A.data_ptr(), B.data_ptr(), out.data_ptr(), M, N, K, int(bool(split)),
                                      _lib.stream_ptr()), "nce_tc_gemm")
    return out


class NCEModel:
    """Geometry + parameters of one cell, uploaded to the device (``nce_nce_create``)."""

    def __init__(self, cs, structure, params, mu=None, sd=None, shell_edges=(0.0, 3.3), act="tanh", pool="mean",
                 ys=1.0, ym=0.0, mma=0, geo=None):
        depth = len(params["layers"])
        # 0 float32 CUDA cores; bf16 / split-bf16 tensor cores: 1 / 3 mma.sync, 2 / 4 tcgen05 (tensor memory)
        self.mma = int(mma)
        self.cs, self.params, self.act, self.pool = cs, params, act, pool
        # geo: the geometry of another model of the same cell, cluster space, shells and depth (an ensemble's seeds)
        self.geo = geo = geo if geo is not None else build_geometry(cs, structure, list(shell_edges), depth)
        K1 = geo["K"] + 1
        self.mu = np.zeros(K1) if mu is None else np.asarray(mu, float)
        self.sd = np.ones(K1) if sd is None else np.asarray(sd, float)
        self.ys, self.ym = float(ys), float(ym)
        self.depth = depth
        self.N, self.nA = geo["N"], geo["nA"]
        self.C0 = K1
        self.D = params["layers"][0]["self"].shape[1] if depth else 16
        self.norm = float(self.nA) if pool == "mean" else 1.0
        self.scale_eV = self.ys * self.N if pool == "mean" else 1.0
        self.perm, self.inv_perm = geo["perm"], geo["inv_perm"]
        self.sig0 = geo["sig"]
        self._build_desc()
        self._handle = None

    def _build_desc(self):
        g = self.geo; keep = self.keep = {}
        a = lambda name, x, dt: keep.__setitem__(name, np.ascontiguousarray(np.asarray(x, dt))) or keep[name]
        nB, J, mo, P, W = g["nB"], g["J"], g["mo"], g["P"], g["W"]
        a("Rv_b", g["Rv_b"], np.int32); a("Rv_uo", g["Rv_uo"], np.int32); a("Rv_p", g["Rv_p"], np.int32)
        a("Rv_col", g["Rv_col"], np.int32); a("Rv_m", g["Rv_m"], np.uint8)
        col = g["Rv_col"]
        w = np.where(g["Rv_v"], g["nA"] / (g["Rv_ord"] * g["norm"][col] * self.sd[col + 1]), 0.0)
        a("Rv_w", w, np.float64)
        a("Mb", g["Mb"], np.int32); th = a("theta", g["theta"], np.float64)
        a("Sh_b", g["Sh_b"], np.int32); a("Sh_uo", g["Sh_uo"], np.int32); a("Sh_m", g["Sh_m"], np.uint8)
        a("Sh_inv", 1.0 / np.maximum(g["Sh_m"].sum(-1), 1), np.float32)
        # receptive-field offsets ordered by the level where they first appear
        L = self.depth
        lists, ends = [], []
        for b in range(nB):
            seen = set(); order = []; e = []
            for l in range(L + 1):
                n = int(g["ball_n"][l][b])
                for bb, o in zip(g["ball_b"][l][b][:n], g["ball_off"][l][b][:n]):
                    it = (int(bb), tuple(int(x) for x in o))
                    if it not in seen:
                        seen.add(it); order.append(it)
                e.append(len(order))
            lists.append(order); ends.append(e)
        wL = max(len(o) for o in lists)
        bb_ = np.zeros((nB, wL), np.int32); bo = np.zeros((nB, wL, 3), np.int64)
        for b in range(nB):
            bb_[b] = b
            for q, (x, o) in enumerate(lists[b]):
                bb_[b, q] = x; bo[b, q] = o
        U, d = g["U"], g["d"]
        a("ball_b", bb_, np.int32); a("ball_uo", np.mod(bo @ U.T, d), np.int32); a("ball_end", np.array(ends), np.int32)
        # each masked reverse-row member as an index into its site's ball-0 list
        rloc = np.zeros((nB, J, mo), np.uint16)
        for b in range(nB):
            pos0 = {it: q for q, it in enumerate(lists[b][:ends[b][0]])}
            for jj in range(J):
                for mm in range(mo):
                    if g["Rv_m"][b, jj, mm] and g["Rv_v"][b, jj]:
                        rloc[b, jj, mm] = pos0[(int(g["Rv_b"][b, jj, mm]), tuple(int(x) for x in g["Rv_off"][b, jj, mm]))]
        a("Rv_loc", rloc, np.uint16)
        self.wL = wL
        p = self.params
        a("lin", p["lin"], np.float32)
        a("head_w", p["head"]["w"] if self.depth else np.zeros(16), np.float32)
        a("mu", self.mu, np.float32); a("sd", self.sd, np.float32)
        gate = bool(self.depth and "gate" in p["layers"][0])
        for l, Ly in enumerate(p["layers"]):
            a(f"W{l}", np.concatenate([Ly["self"]] + [Ly["shell"][q] for q in range(Ly["shell"].shape[0])], axis=0), np.float32)
            a(f"b{l}", Ly["b"], np.float32)
            if gate:
                a(f"G{l}", np.concatenate([Ly["gate"][q] for q in range(Ly["gate"].shape[0])], axis=0), np.float32)
                a(f"gb{l}", Ly["gb"], np.float32)
        a("act_b", g["grp_b"], np.int32); nb = a("act_nb", g["grp_nb"], np.int32)
        cum = np.floor(np.cumsum(nb) / nb.sum() * 2.0 ** 32).astype(np.uint64); cum[-1] = np.uint64(2 ** 32)
        a("grp_cum", cum, np.uint64)
        s = _lib.NceNceDesc()
        s.nB, s.J, s.mo, s.P, s.W, s.depth, s.C0, s.D = nB, J, mo, P, W, self.depth, self.C0, self.D
        s.maxM, s.maxP = th.shape[0] - 1, th.shape[1]
        s.wL = wL
        for c in range(3):
            s.d[c] = int(d[c])
        s.n_cells = int(g["n_cells"])
        for f in ("Rv_b", "Rv_uo", "Rv_p", "Rv_col", "Rv_m", "Rv_w", "Mb", "theta", "Sh_b", "Sh_uo", "Sh_m", "Sh_inv",
                  "ball_b", "ball_uo", "ball_end", "lin", "head_w", "mu", "sd", "act_b", "act_nb", "grp_cum", "Rv_loc"):
            setattr(s, f, keep[f].ctypes.data)
        s.head_b = float(p["head"]["b"])
        for l in range(self.depth):
            s.W_cat[l] = keep[f"W{l}"].ctypes.data; s.bias[l] = keep[f"b{l}"].ctypes.data
            if gate:
                s.G_cat[l] = keep[f"G{l}"].ctypes.data; s.gate_b[l] = keep[f"gb{l}"].ctypes.data
        s.act = 0 if self.act == "tanh" else 1
        s.gate = int(gate)
        s.norm = self.norm; s.scale_eV = self.scale_eV
        s.mma = self.mma
        s.n_groups, s.max_gb = keep["act_b"].shape
        self.desc = s

    @property
    def handle(self):
        if self._handle is None:
            h = C.c_void_p()
            _lib.check(_lib.lib().nce_nce_create(C.byref(self.desc), C.byref(h)), "nce_nce_create")
            self._handle = h
        return self._handle

    def check_errors(self):
        """Raise NceError if a kernel on this model flagged an error since the last check (and clear the flags)."""
        _lib.raise_device_errors(_lib.lib().nce_nce_errors, self.handle, _lib.NCE_ERROR_FLAGS, "NeuralCE kernels")

    def close(self):
        if self._handle is not None:
            _lib.lib().nce_nce_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NCEState:
    """Device PT state of R replicas (torch buffers) in the C-ABI layout."""

    def __init__(self, model: NCEModel, sigma, beta_slot, ladder_id=None, device="cuda"):
        import torch
        R, N = sigma.shape
        self.R, self.N, self.model = R, N, model
        f32 = dict(dtype=torch.float32, device=device)
        self.sigma = torch.as_tensor(np.ascontiguousarray(sigma), dtype=torch.int8).to(device)
        self.h0 = torch.zeros((R, N, model.C0), **f32)
        self.hmid = torch.zeros((max(model.depth - 1, 0), R, N, model.D), **f32) if model.depth >= 2 else None
        self.e = torch.zeros((R, N), **f32)
        self.E = torch.zeros(R, dtype=torch.float64, device=device)
        self.beta_slot = torch.as_tensor(np.asarray(beta_slot, np.float32)).to(device)
        self.rep_of_slot = torch.arange(R, dtype=torch.int32, device=device)
        self.slot_of_rep = torch.arange(R, dtype=torch.int32, device=device)
        self.ladder_id = torch.as_tensor(np.zeros(R, np.int32) if ladder_id is None else np.asarray(ladder_id, np.int32)).to(device)
        self.n_acc = torch.zeros(R, dtype=torch.int64, device=device)
        self.n_ex = torch.zeros(1, dtype=torch.int64, device=device)
        self.n_near = torch.zeros(R, dtype=torch.int64, device=device)   # near-threshold Metropolis steps

    def struct(self):
        s = _lib.NceNceState()
        s.R, s.N = self.R, self.N
        for f in ("sigma", "h0", "e", "E", "beta_slot", "rep_of_slot", "slot_of_rep", "ladder_id", "n_acc", "n_ex", "n_near"):
            setattr(s, f, getattr(self, f).data_ptr())
        s.hmid = self.hmid.data_ptr() if self.hmid is not None else None
        return s

    def full_cache(self, stream=None):
        st = self.struct()
        _lib.check(_lib.lib().nce_nce_full_cache(self.model.handle, C.byref(st), _lib.stream_ptr(stream)), "nce_nce_full_cache")
        return self

    def run_chunk(self, n_steps, step0, seed=0, proposals=None, sample_interval=1, E_samples=None, dE_out=None, force=0,
                  exchange_rounds=0, ex_parity=0, ex_u=None, stream=None, cluster=1, ctas_per_sm=1, near_eV=0.0):
        c = _lib.NceNceChunk()
        c.n_steps, c.step0, c.seed = int(n_steps), int(step0), int(seed) & 0xFFFFFFFFFFFFFFFF
        if proposals is not None:
            c.prop_a, c.prop_b, c.prop_u = (_lib.ptr(p) for p in proposals)
        c.sample_interval = int(sample_interval); c.E_samples = _lib.ptr(E_samples); c.dE_out = _lib.ptr(dE_out)
        c.force = int(force); c.exchange_rounds = int(exchange_rounds); c.ex_parity = int(ex_parity); c.ex_u = _lib.ptr(ex_u)
        c.cluster = int(cluster); c.ctas_per_sm = int(ctas_per_sm); c.near_eV = float(near_eV)
        st = self.struct()
        _lib.check(_lib.lib().nce_nce_run_chunk(self.model.handle, C.byref(st), C.byref(c), _lib.stream_ptr(stream)),
                   "nce_nce_run_chunk")


class NCEPatch:
    """What ``local_delta`` returns as the reference's patch: the swap kept on the device for ``commit``.  It is valid
    until the next call that runs steps on the same models (the engine keeps one evaluated swap per replica)."""

    def __init__(self, cache, serial, i, j):
        self.cache, self.serial, self.i, self.j = cache, serial, int(i), int(j)


class NCECache:
    """The reference's ``full_cache`` result on the device: one ``NCEState`` per model of the ensemble (one model
    unless seed_idx < 0), each with its own layer-0 / hidden / site-energy caches and occupancy."""

    def __init__(self, states):
        self.states = states
        self.serial = 0

    @property
    def sigma(self):
        return self.states[0].sigma[0]

    @property
    def E(self):
        """energy in the model's standardised units, mean over the ensemble (device float64, per replica)"""
        return sum(s.E for s in self.states) / len(self.states)


class EnsembleState:
    """R replicas of an ensemble of models (the reference's seed_idx < 0: energies and dE are the means over the trained
    seeds, ``neuralce/nce/mc_model.py:181-188``), with the ``NCEState`` interface the drivers use.  Each model keeps
    its own caches of the same occupancies; a step evaluates the swap on every model (``nce_nce_local_delta``), decides
    on the mean dE (``nce_nce_accept``) and commits the decision on every model (``nce_nce_commit``), all on the
    device.  Proposals and uniforms are the chunk kernels' (Philox keyed by seed, global step and temperature slot);
    exchanges use the mean energies with the kernels' exchange counters."""

    def __init__(self, models, sigma, beta_slot, ladder_id=None):
        self.models = models
        self.states = [NCEState(m, sigma, beta_slot, ladder_id) for m in models]
        self.model = models[0]
        s0 = self.states[0]
        self.R, self.N = s0.R, s0.N
        self.beta_slot, self.ladder_id = s0.beta_slot, s0.ladder_id

    sigma = property(lambda self: self.states[0].sigma)
    rep_of_slot = property(lambda self: self.states[0].rep_of_slot)
    slot_of_rep = property(lambda self: self.states[0].slot_of_rep)
    n_acc = property(lambda self: self.states[0].n_acc)
    n_ex = property(lambda self: self.states[0].n_ex)
    n_near = property(lambda self: self.states[0].n_near)

    @property
    def E(self):
        return sum(s.E for s in self.states) / len(self.states)

    def broadcast(self):
        """copy the first model's occupancies, slots and counters to the others (after a restore)"""
        for s in self.states[1:]:
            for f in ("sigma", "rep_of_slot", "slot_of_rep", "n_acc", "n_ex"):
                getattr(s, f).copy_(getattr(self.states[0], f))
        return self

    def full_cache(self, stream=None):
        for s in self.states:
            s.full_cache(stream)
        return self

    def check_errors(self):
        for m in self.models:
            m.check_errors()

    def run_chunk(self, n_steps, step0, seed=0, sample_interval=1, E_samples=None, exchange_rounds=0, **_):
        import torch
        from .dist import exchange_slots
        R, S, dev = self.R, len(self.models), self.sigma.device
        i, j, u = proposal_block(self.model, seed, step0, n_steps, self.slot_of_rep.cpu().numpy())
        pa, pb = torch.as_tensor(i, device=dev), torch.as_tensor(j, device=dev)
        pu = torch.as_tensor(u, device=dev)
        dE = torch.empty((S, R), dtype=torch.float64, device=dev)
        acc = torch.empty(R, dtype=torch.int32, device=dev)
        L = _lib.lib(); sp = _lib.stream_ptr()
        structs = [C.byref(st.struct()) for st in self.states]
        s0 = self.states[0]
        for k in range(int(n_steps)):
            for q, (m, st) in enumerate(zip(self.models, structs)):
                _lib.check(L.nce_nce_local_delta(m.handle, st, pa[k].data_ptr(), pb[k].data_ptr(), dE[q].data_ptr(), sp),
                           "nce_nce_local_delta")
            _lib.check(L.nce_nce_accept(dE.data_ptr(), S, R, self.model.scale_eV, s0.beta_slot.data_ptr(),
                                        s0.slot_of_rep.data_ptr(), pu[k].data_ptr(), acc.data_ptr(), sp), "nce_nce_accept")
            for m, st in zip(self.models, structs):
                _lib.check(L.nce_nce_commit(m.handle, st, acc.data_ptr(), sp), "nce_nce_commit")
            if E_samples is not None and (k + 1) % sample_interval == 0:
                E_samples[(k + 1) // sample_interval - 1] = self.E[self.rep_of_slot.long()]
        if exchange_rounds and R > 1:
            E_eV = self.E.cpu().numpy() * self.model.scale_eV
            ros = self.rep_of_slot.cpu().numpy().astype(np.int64)
            lid = self.ladder_id.cpu().numpy(); beta = self.beta_slot.cpu().numpy()
            n_ex = 0
            for q in range(int(exchange_rounds)):
                ros, n = exchange_slots(E_eV, beta, lid, ros, seed, int(step0) + int(n_steps), q)
                n_ex += n
            sor = np.empty(R, np.int64); sor[ros] = np.arange(R)
            for st in self.states:
                st.rep_of_slot.copy_(torch.as_tensor(ros.astype(np.int32), device=dev))
                st.slot_of_rep.copy_(torch.as_tensor(sor.astype(np.int32), device=dev))
                st.n_ex += n_ex
        return self


def _swap_of(sig, flips):
    """(i, j) of a swap written as the reference's flips [[i, sig[j]], [j, sig[i]]]; anything else is refused."""
    f = np.asarray(flips.cpu() if hasattr(flips, "cpu") else flips, np.int64).reshape(-1, 2)
    if f.shape[0] != 2:
        raise ValueError("this engine evaluates swaps: flips must be [[i, sig[j]], [j, sig[i]]]")
    (i, si), (j, sj) = (int(x) for x in f[0]), (int(x) for x in f[1])
    get = (lambda k: int(sig[k].item())) if hasattr(sig, "device") else (lambda k: int(np.asarray(sig)[k]))
    if si != get(j) or sj != get(i):
        raise ValueError("this engine evaluates swaps: flips must be [[i, sig[j]], [j, sig[i]]]")
    return i, j


def _philox_np(c0, c1, c2, c3, k0, k1):
    """Philox4x32-10 on uint64 arrays holding 32-bit words (the counter-based generator the kernels use)."""
    M = np.uint64(0xFFFFFFFF)
    c0, c1, c2, c3 = (np.asarray(x, np.uint64) & M for x in (c0, c1, c2, c3))
    k0, k1 = np.uint64(k0) & M, np.uint64(k1) & M
    for rnd in range(10):
        if rnd:
            k0 = (k0 + np.uint64(0x9E3779B9)) & M; k1 = (k1 + np.uint64(0xBB67AE85)) & M
        p0 = np.uint64(0xD2511F53) * c0; p1 = np.uint64(0xCD9E8D57) * c2
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ k0) & M, p1 & M, ((p0 >> np.uint64(32)) ^ c3 ^ k1) & M, p0 & M
    return c0, c1, c2, c3


def proposal_block(model, seed, step0, n_steps, slots):
    """The chunk kernels' proposals and uniforms for global steps step0 .. step0 + n_steps - 1 of the given temperature
    slots (Philox counters (step, slot), key = seed): (i, j) int32 and u float64, each (n_steps, len(slots))."""
    slots = np.asarray(slots, np.uint64)
    g = (np.uint64(step0) + np.arange(n_steps, dtype=np.uint64))[:, None] * np.ones(len(slots), np.uint64)[None]
    t = np.broadcast_to(slots[None], g.shape)
    k0, k1 = int(seed) & 0xFFFFFFFF, (int(seed) >> 32) & 0xFFFFFFFF
    lo, hi = g & np.uint64(0xFFFFFFFF), g >> np.uint64(32)
    x = _philox_np(lo, hi, t, 0, k0, k1)
    act_b, act_nb, cum = model.keep["act_b"], model.keep["act_nb"].astype(np.uint64), model.keep["grp_cum"]
    grp = np.zeros(g.shape, np.int64); ba = np.zeros(g.shape, np.uint64); bb = np.zeros(g.shape, np.uint64)
    if len(act_nb) > 1 or act_nb[0] > 1:
        y = _philox_np(lo, hi, t, 1, k0, k1)
        for q in range(len(act_nb) - 1):
            grp += (y[0] >= np.uint64(cum[q])) & (grp == q)
        nb = act_nb[grp]
        ba, bb = (y[1] * nb) >> np.uint64(32), (y[2] * nb) >> np.uint64(32)
    n_cells, nB = np.uint64(int(model.desc.n_cells)), int(model.desc.nB)
    i = ((x[0] * n_cells) >> np.uint64(32)).astype(np.int64) * nB + act_b[grp, ba.astype(np.int64)]
    j = ((x[1] * n_cells) >> np.uint64(32)).astype(np.int64) * nB + act_b[grp, bb.astype(np.int64)]
    m = (x[2] << np.uint64(21)) | (x[3] >> np.uint64(11))
    u = (m + np.uint64(1)).astype(np.float64) * 2.0 ** -53
    return i.astype(np.int32), j.astype(np.int32), u


def propose_sites(model, key):
    """The engine's O(1) swap proposal (``gpu_layer0_implicit.py:205-218``): sublattice group by size, uniform cell
    and basis site of the group, twice.  key = (seed, step, slot) or an int seed (step 0, slot 0): the same
    Philox4x32-10 draw the chunk kernels make for that slot at that step.  Returns (i, j) in canonical order."""
    seed, g, t = (int(key), 0, 0) if np.ndim(key) == 0 else (int(k) for k in key)
    d = model.desc
    k = [seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF]
    x = _lib.philox4x32([g & 0xFFFFFFFF, (g >> 32) & 0xFFFFFFFF, t, 0], k)
    act_b, act_nb, cum = model.keep["act_b"], model.keep["act_nb"], model.keep["grp_cum"]
    grp, ba, bb = 0, 0, 0
    if len(act_nb) > 1 or act_nb[0] > 1:
        y = _lib.philox4x32([g & 0xFFFFFFFF, (g >> 32) & 0xFFFFFFFF, t, 1], k)
        while len(act_nb) > 1 and grp < len(act_nb) - 1 and y[0] >= int(cum[grp]):
            grp += 1
        ba, bb = (y[1] * int(act_nb[grp])) >> 32, (y[2] * int(act_nb[grp])) >> 32
    n_cells, nB = int(d.n_cells), int(d.nB)
    i = ((x[0] * n_cells) >> 32) * nB + int(act_b[grp, ba])
    j = ((x[1] * n_cells) >> 32) * nB + int(act_b[grp, bb])
    return i, j


def setup(mdl, atoms: Structure, seed_idx=0, dtype="float32", table=None, mma=0):
    """Reference-shaped entry (``mc_model.py:60-111,175-228``): the MC machinery for ``atoms`` on the GPU.

    Returns the reference's keys: ``energy(sig)`` (eV/atom), ``full_cache(sig)`` -> cache, ``local_delta(cache, sig,
    flips)`` -> (dE_std, patch, sig), ``commit(cache, patch, accept)`` -> cache, ``propose(key)`` -> (i, j),
    ``energy_of(cache)``, ``perm`` / ``inv_perm``, ``to_eV_per_atom``, ``dE_eV_total``, ``sig0`` (canonical order).
    ``local_delta`` / ``commit`` run on the device through ``nce_nce_local_delta`` / ``nce_nce_commit``; flips must
    be a swap ([[i, sig[j]], [j, sig[i]]], the only move of the reference's NeuralCE driver).  seed_idx < 0: the
    ensemble of every trained seed, energies and dE the mean over the seeds (``mc_model.py:181-188``)."""
    import torch
    if table not in (None, "implicit"):
        raise ValueError("only the implicit (template-only) geometry is implemented on this engine")
    if dtype not in ("float32", None):
        raise ValueError("the engine's NCE path computes in float32 (the oracle is the float64 reference)")
    if int(mdl.get("spin", 0) or 0):
        raise NotImplementedError("spin models are not on this engine's path")
    cs = ClusterSpace.build(mdl["primitive"], list(mdl["cutoffs"]))
    seeds = list(range(len(mdl["params"]))) if seed_idx is not None and int(seed_idx) < 0 else [int(seed_idx or 0)]
    models, Ps = [], []
    geo = None
    for k in seeds:
        P, mu, sd = expand_params(mdl, k)
        m = NCEModel(cs, atoms, P, mu, sd, shell_edges=list(mdl["shell_edges"]), act="tanh", pool="mean",
                     ys=mdl["ys"], ym=mdl["ym"], mma=mma, geo=geo)
        geo = m.geo
        models.append(m); Ps.append(P)
    model = models[0]
    ys, ym, n_atoms = mdl["ys"], mdl["ym"], len(atoms)
    one = np.ones(1, np.float32)

    def full_cache(sig, spin_state=None):
        sig = np.asarray(sig.cpu() if hasattr(sig, "cpu") else sig, np.int8)[None]
        return NCECache([NCEState(m, sig, one).full_cache() for m in models])

    def energy_of(cache, P=None):
        return float(cache.E[0].item())

    def energy(sig, spin_state=None):
        return energy_of(full_cache(sig)) * ys + ym

    def local_delta(cache, sig, flips, spin_state=None, sflips=None):
        if spin_state is not None or sflips is not None:
            raise NotImplementedError("spin models are not on this engine's path")
        i, j = _swap_of(sig, flips)
        dev = cache.states[0].sigma.device
        pa = torch.tensor([i], dtype=torch.int32, device=dev); pb = torch.tensor([j], dtype=torch.int32, device=dev)
        dE = torch.empty((len(models), 1), dtype=torch.float64, device=dev)
        for k, (m, st) in enumerate(zip(models, cache.states)):
            _lib.check(_lib.lib().nce_nce_local_delta(m.handle, C.byref(st.struct()), pa.data_ptr(), pb.data_ptr(),
                                                      dE[k].data_ptr(), _lib.stream_ptr()), "nce_nce_local_delta")
        cache.serial += 1
        for m in models:
            m.last_eval = (id(cache), cache.serial)
        return dE.mean(0)[0], NCEPatch(cache, cache.serial, i, j), sig

    def commit(cache, patch, accept):
        if patch.cache is not cache or any(getattr(m, "last_eval", None) != (id(cache), patch.serial) for m in models):
            raise RuntimeError("commit: this patch is no longer held by the engine (another local_delta or chunk ran "
                               "on the same models since)")
        dev = cache.states[0].sigma.device
        acc = accept.to(device=dev, dtype=torch.int32).reshape(1) if hasattr(accept, "to") else \
            torch.tensor([int(bool(accept))], dtype=torch.int32, device=dev)
        for m, st in zip(models, cache.states):
            _lib.check(_lib.lib().nce_nce_commit(m.handle, C.byref(st.struct()), acc.data_ptr(), _lib.stream_ptr()),
                       "nce_nce_commit")
            m.last_eval = None
        return cache

    return dict(cs=cs, P=Ps[0], Ps=Ps, model=model, models=models, depth=model.depth, ym=ym, ys=ys, n_atoms=n_atoms,
                n_active=model.nA, sig0=model.sig0, energy=energy, full_cache=full_cache, energy_of=energy_of,
                F=dict(energy_of=energy_of), local_delta=local_delta, commit=commit,
                propose=lambda key: propose_sites(model, key), perm=model.perm, inv_perm=model.inv_perm, implicit=True,
                geo=model.geo, ensemble=len(models) > 1,
                to_eV_per_atom=lambda E_std: E_std * ys + ym, dE_eV_total=lambda dE_std: dE_std * ys * n_atoms,
                new_state=lambda sig, betas: (EnsembleState(models, np.asarray(sig, np.int8), betas) if len(models) > 1
                                              else NCEState(model, np.asarray(sig, np.int8), betas)))
