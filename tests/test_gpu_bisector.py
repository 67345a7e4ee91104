"""Bisector injection on the GPU (soapgb_bisector_inject) against the reference's own
functions (golden vectors, bit for bit) and against the numpy restatement on a
full-size seed spectrum (310,000 px, 20 mu bins)."""
import os

import numpy as np
import pytest

import oracle
from soap_gpu_gb300 import synth
from soap_gpu_gb300.api import SoapError

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_bis.npz"))


@pytest.mark.parametrize("device_mode", [False, True])
def test_injection_matches_reference(ctx, device_mode):
    torch = pytest.importorskip("torch")
    conv = (lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")) if device_mode else (lambda a: a)
    back = (lambda t: t.cpu().numpy()) if device_mode else (lambda a: a)
    w, f, sc = conv(GOLD["wave"]), conv(GOLD["flux"]), float(GOLD["scale"])
    q = back(ctx.bisector_inject(w, f, conv(GOLD["q_coeffs"]), scale=sc))
    a = back(ctx.bisector_inject(w, f, conv(GOLD["up"]), conv(GOLD["low"]), conv(GOLD["dep_cut"]),
                                 conv(GOLD["vcut"]), conv(GOLD["vshift"]), scale=sc))
    if device_mode:
        ctx.synchronize()
    assert np.array_equal(q, GOLD["quiet"])
    assert np.array_equal(a, GOLD["active"])


def test_injection_full_size(ctx):
    case = synth.make_case(1)
    rng = np.random.default_rng(5)
    wave = case.lambda0 + np.arange(case.n) * case.step
    flux = synth._line_spectrum(wave, np.sort(rng.uniform(wave[50], wave[-50], 6000)),
                                rng.uniform(0.05, 0.9, 6000), rng.uniform(0.03, 0.08, 6000), case.lambda0, case.step)
    coeffs = rng.uniform(-300.0, 300.0, (case.n_mu, 4))
    got = ctx.bisector_inject(wave, flux, coeffs, scale=1.0)
    ref = oracle.bisector_inject(wave, flux, 0, coeffs, scale=1.0)
    assert np.array_equal(got, ref)


def test_folded_grid_reports_status(ctx):
    # a velocity polynomial steep enough to fold the shifted grid: the kernels' own
    # order check turns it into an error, the call returns normally
    with pytest.raises(SoapError, match="status 61"):
        ctx.bisector_inject(GOLD["wave"], GOLD["flux"], np.array([[3e7, 0.0, 0.0, 0.0]]), scale=1.0)
    # the context stays usable
    q = ctx.bisector_inject(GOLD["wave"], GOLD["flux"], GOLD["q_coeffs"], scale=float(GOLD["scale"]))
    assert np.array_equal(q, GOLD["quiet"])


@pytest.mark.parametrize("side_stream", [False, True])
def test_device_calls_follow_the_torch_stream(ctx, side_stream):
    # the input is written on torch's current stream behind a long spin, and the result
    # read there, with no synchronisation in between: a call that ran on a stream of its
    # own would read the input before the copy or be read before it finished
    torch = pytest.importorskip("torch")
    dev = "cuda:0"
    w = torch.as_tensor(GOLD["wave"], device=dev)
    c = torch.as_tensor(GOLD["q_coeffs"], device=dev)
    src = torch.as_tensor(GOLD["flux"], device=dev)
    f = torch.zeros_like(src)
    s = torch.cuda.Stream() if side_stream else torch.cuda.default_stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        for _ in range(3):
            f.zero_()
            torch.cuda._sleep(50_000_000)   # about 25 ms of spinning on this stream
            f.copy_(src)
            q = ctx.bisector_inject(w, f, c, scale=float(GOLD["scale"]))
            got = torch.empty(q.shape, dtype=q.dtype, pin_memory=True)
            got.copy_(q, non_blocking=True)
            s.synchronize()
            assert np.array_equal(got.numpy(), GOLD["quiet"])
