"""The allocation-free convolution entry point, through the C ABI.

soapgb_lower_resolution_noalloc exists for callers that must not have the library
allocate device memory (their device memory is owned by another allocator, or a
cudaMalloc / cudaFree pair would stall a latency-bound loop).  It keeps its scratch
in a fixed array inside the library; these tests check that two consecutive calls
give the same result as the allocating soapgb_lower_resolution (same PLAIN64
arithmetic: the tolerance of the PLAIN64 parity tests), that a request of exactly
soapgb_noalloc_capacity(n_eff) spectra is accepted and one more is refused, and that
the call leaves the calling thread's current device as it found it.  This file is
collected last so that a failure here never hides another test's result.
"""
import ctypes

import numpy as np
import pytest

from _cases import small_inputs

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the PLAIN64 tolerance of test_gpu_parity.py


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    from soap_gpu_gb300 import _lib
    from soap_gpu_gb300.api import Context, torch_stream_handle

    L = _lib.load()
    inp = small_inputs()
    n, n_eff = inp.wave.size, 4096
    rng = np.random.default_rng(17)
    base = np.zeros(n)
    base[:n_eff] = 800.0 * inp.q_sed[0, :n_eff]
    spec = np.zeros((3, n))
    spec[:, :n_eff] = 40.0 * rng.uniform(0, 1, (3, n_eff)) * inp.q_norm[2, :n_eff]
    dev = "cuda:0"
    wave_d = torch.as_tensor(inp.wave, device=dev)
    base_d = torch.as_tensor(base, device=dev)
    spec_d = torch.as_tensor(spec, device=dev)
    sigma_v = inp.case.sigma_v
    with Context(0) as ctx:
        stream = ctypes.c_void_p(torch_stream_handle(0))
        assert L.soapgb_set_stream(ctx.h, stream) == 0
        ref = torch.empty((3, n_eff), dtype=torch.float64, device=dev)
        ref_mm = torch.empty((3, 2), dtype=torch.float64, device=dev)
        rc = L.soapgb_lower_resolution(ctx.h, _lib.PLAIN64, n, n_eff, 3, _ptr(wave_d), _ptr(base_d), _ptr(spec_d),
                                       sigma_v, 50.0, 0.005, 0.005, -60000.0, _lib.DEVICE, _ptr(ref), _ptr(ref_mm))
        assert rc == 0, L.soapgb_last_error(ctx.h)
        assert L.soapgb_noalloc_capacity(n_eff) >= 3
        for _ in range(2):   # the second call reuses the array the first one left behind
            out = torch.full((3, n_eff), np.nan, dtype=torch.float64, device=dev)
            mm = torch.full((3, 2), np.nan, dtype=torch.float64, device=dev)
            rc = L.soapgb_lower_resolution_noalloc(ctx.h, n, n_eff, 3, _ptr(wave_d), _ptr(base_d), _ptr(spec_d),
                                                   sigma_v, 50.0, 0.005, 0.005, -60000.0, _ptr(out), _ptr(mm))
            assert rc == 0, L.soapgb_last_error(ctx.h)
            assert L.soapgb_synchronize(ctx.h) == 0
            o, r = out.cpu().numpy(), ref.cpu().numpy()
            assert np.all(np.isfinite(o))
            assert np.max(np.abs(o - r)) <= TOL * np.max(np.abs(r))
            assert np.array_equal(mm.cpu().numpy(), ref_mm.cpu().numpy())


def test_noalloc_rejects_requests_beyond_its_array():
    torch = pytest.importorskip("torch")
    from soap_gpu_gb300 import _lib
    from soap_gpu_gb300.api import Context

    L = _lib.load()
    n_eff = 4096
    cap = int(L.soapgb_noalloc_capacity(n_eff))
    n_spec = cap + 1
    n = 4200
    wave = torch.as_tensor(5000.0 + 0.005 * np.arange(n), device="cuda:0")
    spec = torch.zeros((n_spec, n), dtype=torch.float64, device="cuda:0")
    out = torch.zeros((n_spec, n_eff), dtype=torch.float64, device="cuda:0")
    with Context(0) as ctx:
        rc = L.soapgb_lower_resolution_noalloc(ctx.h, n, n_eff, n_spec, _ptr(wave), None, _ptr(spec), 1107.0, 50.0,
                                               0.005, 0.005, -60000.0, _ptr(out), None)
        assert rc == _lib.ERR_ARG
        assert "scratch" in L.soapgb_last_error(ctx.h).decode()


@pytest.mark.parametrize("n_eff", [1000, 4096, 20480])
def test_noalloc_accepts_exactly_its_capacity(n_eff):
    torch = pytest.importorskip("torch")
    from soap_gpu_gb300 import _lib
    from soap_gpu_gb300.api import Context

    L = _lib.load()
    cap = int(L.soapgb_noalloc_capacity(n_eff))
    assert cap >= 1
    n = n_eff + 160
    dev = "cuda:0"
    wave = torch.as_tensor(5000.0 + 0.005 * np.arange(n), device=dev)
    rng = np.random.default_rng(n_eff)
    row = np.zeros(n)
    row[:n_eff] = rng.uniform(0.0, 0.5, n_eff)
    spec = torch.as_tensor(np.tile(row, (cap, 1)), device=dev)
    out = torch.full((cap, n_eff), np.nan, dtype=torch.float64, device=dev)
    with Context(0) as ctx:
        before = torch.cuda.current_device()
        rc = L.soapgb_lower_resolution_noalloc(ctx.h, n, n_eff, cap, _ptr(wave), None, _ptr(spec), 1107.0, 50.0,
                                               0.005, 0.005, -60000.0, _ptr(out), None)
        assert rc == 0, L.soapgb_last_error(ctx.h)
        assert L.soapgb_synchronize(ctx.h) == 0, L.soapgb_last_error(ctx.h)
        assert torch.cuda.current_device() == before
        o = out.cpu().numpy()
        assert np.all(np.isfinite(o))
        # every row is the same spectrum, so every output row is the first one
        assert np.array_equal(o, np.tile(o[0], (cap, 1)))
