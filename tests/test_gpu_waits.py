"""The bounded waits of the two kernels that stage their inputs by TMA bulk copies
(the persistent integration kernel and the FP32 convolution) run out cleanly.

A context created with SOAPGB_TEST_WAIT_LIMIT (polls per wait) and SOAPGB_TEST_DROP_COPY
in the environment expects the bytes of one staged copy per block but never issues it
(1: the integration kernel's first plan; 2: the convolution's first window; 3: the
integration kernel's first work-unit window, whose wait each thread takes without a
block barrier), so that wait runs out: the kernel records its status word (41 integration, 42
convolution), gives the copies it did issue a bounded wait and returns.  The call
reports the status (soapgb_synchronize: SOAPGB_ERR_DEVICE with the status in the
message), and the GPU stays usable: a fresh context then runs the same call to the
expected result.  No kernel traps, faults or spins without a limit."""
import ctypes

import numpy as np
import pytest

from soap_gpu_gb300 import synth
from soap_gpu_gb300._lib import ERR_DEVICE, SoapError, Star

from _cases import activity

pytestmark = pytest.mark.gpu


def _pipeline(ctx):
    case = synth.small_case(seed=11, grid=48, n=8300, n_phase=6, n_mu=6)
    inp = synth.generate(case)
    n_eff = (case.n // 512) * 512
    maps = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                         inp.mu_boundary, inp.lb)
    cb = dict(q_norm=inp.q_norm, q_sed=inp.q_sed, spot_norm=inp.spot_norm, fac_norm=inp.fac_norm,
              spot_sed=inp.spot_sed[0], fac_sed=inp.fac_sed[0])
    qn = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    qs = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    star = Star(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                (ctypes.c_double * 4)(*inp.lb))
    return ctx.phase_pipeline("fast32", inp.wave, n_eff, star, maps, cb, case.step, activity(case), case.phases,
                              [case.regions for _ in case.phases], qs, qn, case.sigma_v, conv_step=case.step)


@pytest.mark.parametrize("drop,status", [(1, 41), (2, 42), (3, 41)])
def test_staged_copy_wait_runs_out_and_reports(monkeypatch, drop, status):
    from soap_gpu_gb300.api import Context
    with Context(0) as good:
        ref = _pipeline(good)
    monkeypatch.setenv("SOAPGB_TEST_WAIT_LIMIT", "512")
    monkeypatch.setenv("SOAPGB_TEST_DROP_COPY", str(drop))
    bad = Context(0)
    monkeypatch.delenv("SOAPGB_TEST_WAIT_LIMIT")
    monkeypatch.delenv("SOAPGB_TEST_DROP_COPY")
    with pytest.raises(SoapError) as e:
        _pipeline(bad)          # host buffers: the call checks the status word before returning
    assert e.value.code == ERR_DEVICE
    assert "device status %d" % status in str(e.value)
    bad.synchronize()           # the status was cleared when it was reported
    bad.close()
    # the GPU is still usable: a fresh context gives the expected spectra
    with Context(0) as again:
        out = _pipeline(again)
    assert np.array_equal(out, ref)
