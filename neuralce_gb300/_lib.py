"""ctypes binding of libnce_gb300.so (declared in include/nce_gb300.h).

The library is built in-tree by ``neuralce_gb300.build``; ``lib()`` loads it and raises if it is missing, so
no code path silently falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libnce_gb300.so")

i32, i64, u64, f64, f32 = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_float
P = C.POINTER
vp = C.c_void_p


class NceCeTables(C.Structure):
    _fields_ = [("nB", i32), ("J", i32), ("mo", i32), ("n_nbr", i32), ("n_pfc", i32), ("max_sp", i32),
                ("d", i64 * 3), ("n_cells", i64), ("zerolet", f64),
                ("Rv_len", vp), ("Rv_loc", vp), ("Rv_pfc", vp), ("Rv_eci", vp), ("nb_b", vp), ("nb_uo", vp),
                ("Rt", i32), ("T_b", vp), ("T_uo", vp), ("T_pfc", vp), ("T_eci", vp), ("pf", vp),
                ("n_groups", i32), ("max_gb", i32), ("act_b", vp), ("act_nb", vp), ("grp_cum", vp),
                ("Rv_col", vp), ("n_cols", i32), ("Rv_slot", vp)]


class NcePtState(C.Structure):
    _fields_ = [("R", i32), ("N", i64), ("sigma", vp), ("E", vp), ("beta_slot", vp), ("rep_of_slot", vp),
                ("slot_of_rep", vp), ("ladder_id", vp), ("E_min_rep", vp), ("n_acc", vp), ("n_ex", vp), ("cv", vp),
                ("n_near", vp), ("field", vp), ("ex_sync", vp)]


class NcePtChunk(C.Structure):
    _fields_ = [("n_steps", i64), ("step0", i64), ("prop_a", vp), ("prop_b", vp), ("prop_u", vp), ("seed", u64),
                ("sample_interval", i64), ("E_samples", vp), ("do_exchange", i32), ("ex_parity", i32),
                ("ex_u", vp), ("precision", i32), ("warps", i32), ("path", i32), ("cluster", i32), ("step_dev", vp),
                ("near_eV", f64)]


class NceNceDesc(C.Structure):
    _fields_ = [("nB", i32), ("J", i32), ("mo", i32), ("P", i32), ("W", i32), ("depth", i32), ("C0", i32), ("D", i32),
                ("maxM", i32), ("maxP", i32), ("wL", i32), ("d", i64 * 3), ("n_cells", i64),
                ("Rv_b", vp), ("Rv_uo", vp), ("Rv_p", vp), ("Rv_col", vp), ("Rv_m", vp), ("Rv_w", vp),
                ("Mb", vp), ("theta", vp), ("Sh_b", vp), ("Sh_uo", vp), ("Sh_m", vp), ("Sh_inv", vp),
                ("ball_b", vp), ("ball_uo", vp), ("ball_end", vp), ("lin", vp), ("head_w", vp), ("head_b", f64),
                ("W_cat", vp * 4), ("bias", vp * 4), ("G_cat", vp * 4), ("gate_b", vp * 4), ("mu", vp), ("sd", vp),
                ("act", i32), ("gate", i32), ("norm", f64), ("scale_eV", f64),
                ("n_groups", i32), ("max_gb", i32), ("act_b", vp), ("act_nb", vp), ("grp_cum", vp), ("Rv_loc", vp),
                ("mma", i32)]


class NceNceState(C.Structure):
    _fields_ = [("R", i32), ("N", i64), ("sigma", vp), ("h0", vp), ("hmid", vp), ("e", vp), ("E", vp),
                ("beta_slot", vp), ("rep_of_slot", vp), ("slot_of_rep", vp), ("ladder_id", vp), ("n_acc", vp), ("n_ex", vp),
                ("n_near", vp)]


class NceNceChunk(C.Structure):
    _fields_ = [("n_steps", i64), ("step0", i64), ("prop_a", vp), ("prop_b", vp), ("prop_u", vp), ("seed", u64),
                ("sample_interval", i64), ("E_samples", vp), ("dE_out", vp), ("force", i32), ("exchange_rounds", i32),
                ("ex_parity", i32), ("ex_u", vp), ("cluster", i32), ("ctas_per_sm", i32), ("near_eV", f64)]


class NceServerConfig(C.Structure):
    _fields_ = [("hbm_budget", i64), ("max_batch", i32), ("precision", i32), ("warps", i32), ("nce_cluster", i32),
                ("nce_streams", i32), ("starve_s", f64), ("ce_kernel", i32), ("ce_lf_warps", i32)]


class NceJobDesc(C.Structure):
    _fields_ = [("kind", i32), ("model", vp), ("R", i32), ("sigma", vp), ("beta_slot", vp), ("ladder_id", vp),
                ("n_steps", i64), ("exchange_every", i64), ("seed", u64), ("reanchor_chunks", i32),
                ("sigma_out", vp), ("E_out", vp), ("n_acc_out", vp), ("rep_of_slot_out", vp), ("n_ex_out", vp),
                ("flags", i32)]


class NceJobInfo(C.Structure):
    _fields_ = [("status", i32), ("error", i32), ("steps_done", i64), ("n_steps", i64), ("device_bytes", i64),
                ("t_submit", f64), ("t_start", f64), ("t_end", f64)]


class NceServerStats(C.Structure):
    _fields_ = [("queued", i64), ("running", i64), ("done", i64), ("cancelled", i64), ("failed", i64),
                ("bytes_used", i64), ("hbm_budget", i64), ("rounds_ce", i64), ("rounds_nce", i64), ("attempts", i64),
                ("now", f64)]


_lock = threading.Lock()
_lib = None

SIGNATURES = {
    "nce_version": (i32, []),
    "nce_last_error": (i32, [C.c_char_p, C.c_size_t]),
    "nce_ce_create": (i32, [P(NceCeTables), P(vp)]),
    "nce_ce_destroy": (i32, [vp]),
    "nce_ce_energy": (i32, [vp, vp, i32, i32, vp, vp]),
    "nce_ce_delta": (i32, [vp, vp, i32, i32, vp, vp, vp, vp, vp, i32, i32, vp, vp]),
    "nce_ce_run_chunk": (i32, [vp, P(NcePtState), P(NcePtChunk), vp]),
    "nce_ce_cluster_counts": (i32, [vp, vp, i32, vp, vp]),
    "nce_ce_energy_from_counts": (i32, [vp, vp, i32, vp, vp]),
    "nce_ce_run_batch": (i32, [i32, P(vp), P(NcePtState), P(NcePtChunk), vp]),
    "nce_ce_run_chunk_host": (i32, [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, P(NcePtChunk), vp]),
    "nce_ce_errors": (i32, [vp, P(i32)]),
    "nce_ce_field_init": (i32, [vp, vp, i32, vp, vp]),
    "nce_ce_has_local_field": (i32, [vp, P(i32), P(f64)]),
    "nce_pt_minimum": (i32, [P(NcePtState), vp, vp, vp]),
    "nce_philox4x32": (None, [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]),
    "nce_server_create": (i32, [P(NceServerConfig), P(vp)]),
    "nce_server_destroy": (i32, [vp]),
    "nce_job_submit": (i32, [vp, P(NceJobDesc), P(i64)]),
    "nce_job_poll": (i32, [vp, i64, P(NceJobInfo)]),
    "nce_job_cancel": (i32, [vp, i64]),
    "nce_server_query": (i32, [vp, P(NceServerStats)]),
    "nce_job_error": (i32, [vp, i64, C.c_char_p, C.c_size_t]),
    "nce_nce_create": (i32, [P(NceNceDesc), P(vp)]),
    "nce_nce_destroy": (i32, [vp]),
    "nce_nce_full_cache": (i32, [vp, P(NceNceState), vp]),
    "nce_nce_run_chunk": (i32, [vp, P(NceNceState), P(NceNceChunk), vp]),
    "nce_nce_errors": (i32, [vp, P(i32)]),
    "nce_nce_local_delta": (i32, [vp, P(NceNceState), vp, vp, vp, vp]),
    "nce_nce_tc_wait_selftest": (i32, [vp, i32, vp]),
    "nce_nce_commit": (i32, [vp, P(NceNceState), vp, vp]),
    "nce_nce_accept": (i32, [vp, i32, i32, f64, vp, vp, vp, vp, vp]),
    "nce_tc_gemm": (i32, [vp, vp, vp, i32, i32, i32, i32, vp]),
}


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m neuralce_gb300.build` "
                                   "(this package has no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class NceError(RuntimeError):
    pass


def check(rc, what=""):
    if rc != 0:
        buf = C.create_string_buffer(2048)
        lib().nce_last_error(buf, len(buf))
        raise NceError(f"{what}: status {rc}: {buf.value.decode(errors='replace')}")


CE_ERROR_FLAGS = {1: "a proposal index was out of range (the move was rejected)",
                  2: "a delta query was out of range (NaN returned)"}
NCE_ERROR_FLAGS = {1: "a proposal index was out of range", 4: "a receptive field exceeded its tables",
                   8: "a row member was outside the layer-0 ball", 32: "a tensor-core completion wait timed out"}


def raise_device_errors(fn, handle, table, what):
    """Read and clear a model handle's device error word (``nce_ce_errors`` / ``nce_nce_errors``); raise NceError
    naming every flag that was set."""
    f = C.c_int32(0)
    check(fn(handle, C.byref(f)), what)
    if f.value:
        names = "; ".join(t for b, t in table.items() if f.value & b) or "unknown flag"
        raise NceError(f"{what}: device error flags 0x{f.value:x}: {names}")


def ptr(x):
    """device/host address of a torch tensor or numpy array (None -> NULL)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    raise TypeError(type(x))


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def philox4x32(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().nce_philox4x32(c, k, o)
    return [int(x) for x in o]
