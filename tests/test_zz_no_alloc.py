"""nce_ce_energy_noalloc: the full-energy entry point for callers that cannot allocate device memory while they
run (their device memory is reserved up front by their own pool, or cudaMalloc's implicit synchronisation is
not acceptable in their loop).  Its scratch is a fixed array inside the library; this test checks, through the
C ABI, that two calls in a row give the same energies as nce_ce_energy (which allocates its scratch), within
the float64 tolerance of the other energy tests, and that requests beyond the array's limit are refused.

Collected last on purpose (file name), so a run that stops at the first failure has run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fn():
    from neuralce_gb300 import _lib
    L = _lib.lib()
    f = L.nce_ce_energy_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    return f


@pytest.mark.parametrize("precision", [64, 32])
def test_noalloc_energy_matches_energy_two_calls(cuda, precision):
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.workloads import ce_config, replica_configs
    f = _fn()
    gce, sig = ce_config(8, seed=4)
    batches = [replica_configs(sig, 6, 11), replica_configs(sig, 3, 12)]
    for sig_r in batches:                                   # two calls in a row, different inputs
        sd = torch.as_tensor(sig_r).cuda()
        want = gce.batched_energy(sd, precision=precision).cpu().numpy()
        out = torch.full((len(sig_r),), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(f(gce.handle, sd.data_ptr(), len(sig_r), precision, out.data_ptr(), _lib.stream_ptr()),
                   "nce_ce_energy_noalloc")
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        tol = 1e-10 if precision == 64 else 1e-5
        assert np.all(np.isfinite(got))
        assert np.abs(got - want).max() <= tol * max(1.0, np.abs(want).max()), (got, want)


def test_noalloc_energy_at_the_limit(cuda):
    """65,535 configurations (the documented maximum) of a 16-site cell run and match nce_ce_energy."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.workloads import ce_config
    f = _fn()
    gce, sig = ce_config(2, seed=0)
    R = 65535
    rng = np.random.default_rng(5)
    sig_r = np.stack([sig[rng.permutation(len(sig))] for _ in range(64)]).astype(np.int8)
    sig_r = np.ascontiguousarray(np.tile(sig_r, (R // 64 + 1, 1))[:R])
    sd = torch.as_tensor(sig_r).cuda()
    want = gce.batched_energy(sd).cpu().numpy()
    out = torch.full((R,), float("nan"), dtype=torch.float64, device="cuda")
    _lib.check(f(gce.handle, sd.data_ptr(), R, 64, out.data_ptr(), _lib.stream_ptr()), "nce_ce_energy_noalloc")
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert np.abs(got - want).max() <= 1e-10 * max(1.0, np.abs(want).max())


@pytest.mark.parametrize("R", [65536, 65537])
def test_noalloc_energy_refuses_too_many_configurations(cuda, R):
    torch = cuda
    from neuralce_gb300.workloads import ce_config
    f = _fn()
    gce, _ = ce_config(2, seed=0)
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = f(gce.handle, dummy.data_ptr(), R, 64, dummy.data_ptr(), None)
    assert rc == -1                                          # NCE_ERR_INVALID, nothing launched
