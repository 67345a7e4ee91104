"""Benchmark: phase-spectra/s of the per-phase synthesis path on the 300x300-grid,
310,000-pixel workload (facula + overlapping spot, 100 phases, R = 115000).

One step = the per-phase stages for all 100 phases: region maps, active-region
integration of the tot / flux / bconv deficit spectra, instrumental convolution and
normalisation (SOAP_integration + SOAP_resolution of the reference).  `value` is
phase-spectra/s with the inputs resident in device memory; `e2e` runs the same call
through the C ABI with host buffers (pinned), the host-to-device copy of every input
and the device-to-host copy of the 300 output spectra inside the timed region.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--form fast32|fast64|plain64]
       python bench.py --impl reference ...   (the reference path's CPU restatement,
                                               OpenMP on all host cores)
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spectra/s at 300² grid, 310k px: FP32-comp vs FP64 at ≤1 cm/s RV error"
UNIT = "phase-spectra/s"
C_LIGHT = 299792458.0


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel):
    """Per-launch DRAM traffic (ncu dram__bytes_read.sum + dram__bytes_write.sum) of
    `kernel` from the committed summary profiles/traffic.txt (lines "kernel bytes")."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for ln in f:
            parts = ln.split()
            if len(parts) == 2 and parts[0] == kernel:
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


def rank_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rk = int(os.environ.get("RANK", "0"))
    lr = int(os.environ.get("LOCAL_RANK", str(rk)))
    return ws, rk, lr


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_workload(rank=0, n_phase=100, phase0=0):
    from soap_gpu_gb300 import synth
    case = synth.make_case(1)
    inp = synth.generate(case)
    # weak scaling: every rank integrates its own block of phases of the same star
    phases = (case.phases + rank * case.rot_num)[phase0:phase0 + n_phase]
    return case, inp, phases


def star_struct(case, lb):
    import ctypes
    from soap_gpu_gb300._lib import Star
    return Star(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                (ctypes.c_double * 4)(*lb))


# ---------------------------------------------------------------------------
# own arm
# ---------------------------------------------------------------------------
def run_own(args):
    import torch
    from soap_gpu_gb300._lib import Activity
    from soap_gpu_gb300.api import Context
    from soap_gpu_gb300 import rv

    ws, rk, lr = rank_info()
    dist = ws > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(lr)
    dev = "cuda:%d" % lr
    case, inp, phases = make_workload(rk, args.phases, args.phase0)
    n, n_eff, n_mu = case.n, case.n_eff, case.n_mu
    lb = inp.lb
    star = star_struct(case, lb)
    act = Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, 0)
    regions = [case.regions for _ in phases]
    ctx = Context(lr)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    wave_d = T(inp.wave)
    maps_d = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                           T(inp.mu_boundary), lb)
    cubes_np = dict(q_norm=inp.q_norm, q_sed=inp.q_sed, spot_norm=inp.spot_norm, fac_norm=inp.fac_norm,
                    spot_sed=inp.spot_sed[0], fac_sed=inp.fac_sed[0])
    cubes_d = {k: T(v) for k, v in cubes_np.items()}
    form = args.form
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q_norm_d = ctx.quiet_disk(form, wave_d, cubes_d["q_norm"], n_eff, maps_d, case.grid, case.step)
    q_sed_d = ctx.quiet_disk(form, wave_d, cubes_d["q_sed"], n_eff, maps_d, case.grid, case.step)
    torch.cuda.synchronize()
    quiet_ms = (time.perf_counter() - t0) * 1e3
    phases_d = T(phases)
    out = torch.empty((len(phases), 3, n_eff), dtype=torch.float64, device=dev)

    def step_dev():
        # bulk inputs resident in device memory; the phase and region descriptors (100 +
        # 200 values) stay on the host, so steps queue without a synchronisation
        ctx.phase_pipeline(form, wave_d, n_eff, star, maps_d, cubes_d, case.step, act, phases, regions, q_sed_d,
                           q_norm_d, case.sigma_v, conv_step=case.step, out=out)

    # clocks are sampled from the warm-up on (nvidia-smi needs a moment to start); the
    # warm-up runs at least W steps and at least half a second so the GPU is under load
    clocks = ClockSampler(lr)
    clocks.start()
    tw = time.perf_counter()
    nw = 0
    while nw < args.warmup or time.perf_counter() - tw < 0.5:
        step_dev()
        nw += 1
        if nw % 20 == 0:
            torch.cuda.synchronize()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    l0 = ctx.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step_dev()
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    launches = ctx.launches - l0
    ms = ev0.elapsed_time(ev1)
    if args.profile_only:
        clocks.stop()
        ctx.close()
        return {"profile_only": True, "ms_per_step": ms / args.steps, "launches_per_step": launches / args.steps}
    if dist:
        tdist.barrier()
    clk = clocks.stop()
    t = torch.tensor([ms], device=dev, dtype=torch.float64)
    if dist:
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    ms_total = float(t.item())
    ms_step = ms_total / args.steps
    n_units = len(phases) * ws * args.steps
    value = n_units / (ms_total / 1e3)

    # --- end to end through the C ABI with pinned host buffers ----------------------
    def pinned(a):
        t_ = torch.empty(a.shape, dtype=torch.float64 if a.dtype != np.int32 else torch.int32, pin_memory=True)
        t_.numpy()[...] = a
        return t_.numpy()

    wave_h = pinned(inp.wave)
    cubes_h = {k: pinned(np.ascontiguousarray(v)) for k, v in cubes_np.items()}
    maps_h = {k: pinned(v.cpu().numpy()) for k, v in maps_d.items()}
    qs_h, qn_h = pinned(q_sed_d.cpu().numpy()), pinned(q_norm_d.cpu().numpy())
    ph_h = pinned(phases)
    out_h = pinned(np.zeros((len(phases), 3, n_eff)))
    h2d = (wave_h.nbytes + sum(v.nbytes for v in cubes_h.values()) + sum(v.nbytes for v in maps_h.values()) -
           maps_h["mu"].nbytes + qs_h.nbytes + qn_h.nbytes + ph_h.nbytes)
    # phases without a visible region share one set of rows: it crosses the host link
    # once and the library copies it into the other such phases on host threads
    _, bi_e = ctx.phase_maps(case.grid, case.incl, phases, regions, act)
    n_zero = int(np.count_nonzero(~np.any(bi_e.reshape(len(phases), -1) >= 0, axis=1)))
    row_bytes = 3 * n_eff * 8
    d2h = out_h.nbytes - max(n_zero - 1, 0) * row_bytes

    def step_host():
        ctx.phase_pipeline(form, wave_h, n_eff, star, maps_h, cubes_h, case.step, act, ph_h, regions, qs_h, qn_h,
                           case.sigma_v, conv_step=case.step, out=out_h)

    for _ in range(max(1, args.warmup)):
        step_host()
    if dist:
        tdist.barrier()
    te0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    te = (time.perf_counter() - te0) * 1e3
    te_t = torch.tensor([te], device=dev, dtype=torch.float64)
    if dist:
        tdist.all_reduce(te_t, op=tdist.ReduceOp.MAX)
    e2e_value = n_units / (float(te_t.item()) / 1e3)

    # --- seed preparation: bisector injection of one 20 x 310k cube (CB_injection_faculae) ---
    rng_b = np.random.default_rng(11)
    bis_coeffs = T(rng_b.uniform(-300.0, 300.0, (n_mu, 4)))
    bis_flux = T(inp.q_norm[0])
    for _ in range(2):
        ctx.bisector_inject(wave_d, bis_flux, bis_coeffs)
    torch.cuda.synchronize()
    eb0, eb1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    eb0.record(stream)
    for _ in range(5):
        ctx.bisector_inject(wave_d, bis_flux, bis_coeffs)
    eb1.record(stream)
    eb1.synchronize()
    bis_ms = eb0.elapsed_time(eb1) / 5

    # --- per-kernel CUDA-event times of one step, roofline of the dominant kernel -------
    ctx.trace(True)
    for _ in range(2):
        step_dev()
    ktab = {k: (c / 2.0, ms / 2.0) for k, (c, ms) in ctx.trace_report().items()}
    ctx.trace(False)
    result = None
    if rk == 0:
        peak, peak_kind = measured_peaks()
        dom = max(ktab, key=lambda k: ktab[k][1])
        phases_np = phases_d.cpu().numpy()
        roof = kernel_roofline(dom, ktab, case, phases_np, regions, act, ctx, maps_d, form, dev)
        others = {k: kernel_roofline(k, ktab, case, phases_np, regions, act, ctx, maps_d, form, dev)
                  for k in ("conv32", "norm32", "cube_types") if k in ktab and k != dom}

        # --- the FP64 forms on the same step (the plain form is the reference's arithmetic)
        fp64 = {}
        outs = {}
        for f in ("plain64", "fast64"):
            qn = ctx.quiet_disk(f, wave_d, cubes_d["q_norm"], n_eff, maps_d, case.grid, case.step)
            qs = ctx.quiet_disk(f, wave_d, cubes_d["q_sed"], n_eff, maps_d, case.grid, case.step)
            o_f = torch.empty_like(out)

            def step_f(f=f, qn=qn, qs=qs, o_f=o_f):
                ctx.phase_pipeline(f, wave_d, n_eff, star, maps_d, cubes_d, case.step, act, phases, regions, qs, qn,
                                   case.sigma_v, conv_step=case.step, out=o_f)

            ms_f = timed_steps(step_f, 3, stream)
            fp64[f] = {"value": round(len(phases) / (ms_f / 1e3), 2), "ms_per_step": round(ms_f, 3)}
            outs[f] = (o_f, qs, qn)
        ref_d = outs["plain64"][0]
        fp64["fast32_over_plain64"] = round(value / fp64["plain64"]["value"], 2)
        err = accuracy(ctx, case, inp, out, ref_d)

        # --- the compensated summation variant of the FP32 integration, timed and checked once
        comp = None
        if form == "fast32":
            ctx.set_compensated(False)
            o_c = torch.empty_like(out)

            def step_c():
                ctx.phase_pipeline(form, wave_d, n_eff, star, maps_d, cubes_d, case.step, act, phases, regions,
                                   q_sed_d, q_norm_d, case.sigma_v, conv_step=case.step, out=o_c)

            ms_c = timed_steps(step_c, min(args.steps, 50), stream)
            ctx.trace(True)
            step_c()
            kc = ctx.trace_report()
            ctx.trace(False)
            ctx.set_compensated(True)
            comp = {"summation": "plain FP32 output sums (the timed step uses compensated ones)",
                    "ms_per_step": round(ms_c, 4),
                    "value": round(len(phases) / (ms_c / 1e3), 2),
                    "fir_tile_phase_ms": round(kc.get("fir_tile_phase", (0, 0.0))[1], 4),
                    "accuracy": accuracy(ctx, case, inp, o_c, ref_d)}

        # --- CCF + fit stage (RV series), GPU and the reference's CPU form
        lows = []
        for q in (q_sed_d, q_sed_d, q_norm_d):
            lo, _ = ctx.lower_resolution(form, wave_d, q, n_eff, case.sigma_v, step_mult=case.step,
                                         step_exp=case.step)
            lows.append(lo.reshape(-1))
        quiet_low_d = torch.stack(lows)
        ccf_stage = ccf_fit_stage(ctx, case, inp, out, quiet_low_d, stream)
        if not args.no_cpu:
            ccf_stage["cpu_baseline"] = ccf_fit_cpu(case, inp, ref_d[:2].cpu().numpy())
        cpu = cpu_baseline(case, inp, sample_phases=1) if not args.no_cpu else None
        result = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if form == "fast32" else "f64", "data": "synthetic",
            "config": {"workload": "300x300 grid, 310,000 px (3800-6900 A at 0.01 A), 20 mu bins, facula 3% + "
                                   "spot 1% overlapping, 100 phases per GPU, R=115000",
                       "form": form, "phases_per_step": len(phases), "l2": "inputs (cubes 4x49.6 MB FP64) and "
                       "outputs (744 MB) exceed the 129 MB L2", "quiet_stage_ms": round(quiet_ms, 2),
                       "summation": "FP32 per work unit, unit deficits (about 9 per pixel and tile) added in "
                                    "compensated (Kahan) FP32 sums; the plain-sum variant is timed under "
                                    "'summation_variant'" if form == "fast32" else "FP64"},
            "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "output_bytes_per_step": int(out_h.nbytes),
                    "zero_phases": n_zero,
                    "what": "soapgb_phase_pipeline on pinned host buffers: inputs in, FP64 spectra of every "
                            "phase out; the rows of the phases without a visible region cross the link once "
                            "and are replicated on the host"},
            "gpu_launches": int(launches),
            "roofline": roof,
            "rooflines_other": others,
            "cpu_baseline": cpu,
            "accuracy": err,
            "fp64_forms": fp64,
            "summation_variant": comp,
            "ref_cuda": ref_cuda_record(len(phases)),
            "ccf_fit": ccf_stage,
            "kernels_ms_per_step": {k: round(v[1], 4) for k, v in sorted(ktab.items(), key=lambda x: -x[1][1])},
            "seed_preparation": {"bisector_injection_ms_per_cube": round(bis_ms, 4),
                                 "cube": "%d mu bins x %d px, quiet form, inputs resident" % (n_mu, n)},
            "differentiable": adjoint_timing(ctx, dev),
            "differentiable_shape": diff_batch_timing(ctx, dev, stream, n_star=args.diff_stars)
            if args.diff_stars > 0 else None,
            "batched": batched_timing(ctx, case, inp, wave_d, cubes_d, dev, stream) if not args.no_batch else None,
            "clocks": clk,
        }
    if dist:
        tdist.barrier()
        tdist.destroy_process_group()
    ctx.close()
    return result


def profile_counters(kernel):
    """ncu counters of `kernel` from the committed summary profiles/counters.txt (lines
    "kernel metric value"): the limiter evidence printed beside the roofline."""
    p = os.path.join(ROOT, "profiles", "counters.txt")
    out = {}
    if os.path.exists(p):
        with open(p) as f:
            for ln in f:
                parts = ln.split()
                if len(parts) == 3 and parts[0] == kernel:
                    try:
                        out[parts[1]] = float(parts[2])
                    except ValueError:
                        pass
    return out


def fp32_peak_tflops(dev):
    """Nominal FP32 FMA rate: SMs x 128 lanes x 2 flop x the maximum SM clock
    (MEASURED_PEAKS.json sm_max_mhz, else 2070 MHz)."""
    import torch
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = 2070.0
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    return sms * 128 * 2 * mhz * 1e6 / 1e12


def conv32_flops(case, n_spec):
    """FMA flops the FP32 convolution executes: per spectrum and pixel, 2 flop per tap over
    the reach where the Gaussian weight is at least e^-30 of the centre (the reach of a
    1024-pixel tile is that of its largest sigma, sigma growing with wavelength)."""
    wave = np.arange(case.n_eff) * case.step + case.lambda0
    beta = case.sigma_v / C_LIGHT
    sig = wave * (np.sqrt((1 + beta) / (1 - beta)) - 1) / case.step   # in pixels
    tiles = np.maximum.reduceat(sig, np.arange(0, case.n_eff, 1024))
    reach = np.floor(np.sqrt(60.0) * tiles)
    taps = np.repeat(2 * reach + 1, 1024)[:case.n_eff]
    return float(2.0 * n_spec * taps.sum())


def kernel_roofline(kernel, ktab, case, phases, regions, act, ctx, maps_d, form, dev):
    """Roofline entry of one kernel of the step from its live CUDA-event time.

    fir_tile_phase (active-region integration, all phases in one launch): algorithmic
    bytes per phase (distinct mu rows of its active cells x N_eff x 3 cubes + 2 continua
    + 3 outputs) x sizeof(element).  Those count each phase's read of the cube rows,
    which the kernel serves from L2 across phases, so the DRAM traffic of the ncu capture
    is reported beside them; the kernel is bound by instruction issue (ncu counters).
    conv32: executed FP32 FMA flops against the nominal FP32 rate.  norm32 / cube_types:
    bytes in + out against the measured copy bandwidth."""
    peak, peak_kind = measured_peaks()
    launches, ms = ktab[kernel]
    ms_launch = ms / max(launches, 1.0)
    n_eff, n_phase = case.n_eff, len(phases)
    tsz = 4 if form == "fast32" else 8
    traffic = profile_traffic(kernel)
    counters = profile_counters(kernel)
    if kernel == "fir_tile_phase":
        temp, bi = ctx.phase_maps(case.grid, case.incl, phases, regions, act)
        region = maps_d["region"].cpu().numpy()
        rows = sum(len(np.unique(region[(bi[p] >= -0.5) & (bi[p] <= 1.5)])) for p in range(n_phase))
        b = (rows * 3 + (2 + 3) * n_phase) * n_eff * tsz
        ach = b / (ms_launch / 1e3) / 1e9
        out = {"bound": "issue", "kernel": kernel, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
               "frac": round(ach / peak, 4), "traffic": traffic, "peak_source": peak_kind,
               "algorithmic_bytes_per_launch": int(b),
               "bytes_formula": "sum_p (mu rows touched x 3 cubes + 2 continua + 3 outputs) x N_eff x %d B" % tsz,
               "ms_per_launch": round(ms_launch, 4),
               "bound_evidence": "instruction issue and latency: the cube rows are re-read per phase from L2, "
                                 "DRAM moves far less than the algorithmic bytes (see dram_achieved); ncu counters "
                                 "in counters"}
        if traffic:
            dr = traffic / (ms_launch / 1e3) / 1e9
            out["dram_achieved"] = round(dr, 1)
            out["dram_frac"] = round(dr / peak, 4)
        if counters:
            out["counters"] = counters
        return out
    if kernel == "conv32":
        # phases without a visible region have zero spectra, which the convolution skips
        _, bi = ctx.phase_maps(case.grid, case.incl, phases, regions, act)
        n_spec = 3 * int(np.count_nonzero(np.any(bi.reshape(n_phase, -1) >= 0, axis=1)))
        fl = conv32_flops(case, n_spec)
        pk = fp32_peak_tflops(dev)
        ach = fl / (ms_launch / 1e3) / 1e12
        out = {"bound": "fp32", "kernel": kernel, "achieved": round(ach, 2), "peak": round(pk, 1),
               "unit": "TFLOP/s", "frac": round(ach / pk, 4), "peak_source": "nominal (SMs x 128 x 2 x max clock)",
               "flops_per_launch": fl, "flops_formula": "2 flop x taps within e^-30 of the centre x N_eff x "
               "convolved spectra (%d)" % n_spec, "ms_per_launch": round(ms_launch, 4), "traffic": traffic}
        if counters:
            out["counters"] = counters
        return out
    if kernel == "norm32":
        b = 3 * n_phase * n_eff * (4 + 8)
        formula = "3 n_phase x N_eff x (4 B in + 8 B out)"
    elif kernel == "cube_types":
        b = 4 * case.n_mu * case.n * 8 + 6 * case.n_mu * case.n * 4
        formula = "4 FP64 cubes in + 6 FP32 cubes out, n_mu x N each"
    else:
        return None
    ach = b / (ms_launch / 1e3) / 1e9
    out = {"bound": "hbm", "kernel": kernel, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
           "frac": round(ach / peak, 4), "peak_source": peak_kind, "algorithmic_bytes_per_launch": int(b),
           "bytes_formula": formula, "ms_per_launch": round(ms_launch, 4), "traffic": traffic}
    if counters:
        out["counters"] = counters
    return out


def batched_timing(ctx, case, inp, wave_d, cubes_d, dev, stream, n_star=256, per_batch=64):
    """The batched form on 256 stars of uneven sizes sharing the 310,000-px seeds (grids
    U{100..400}, 1-12 spots and faculae of 0.1-3 % of the hemisphere at latitudes
    U(-60, 60), U{20..200} phases over one rotation, vsini U(1, 10) km/s): every stage
    per star (disk maps, both quiet spectra, lists, plans, integration, convolution,
    normalisation).  The stars run in batches of `per_batch` (the outputs of all 256,
    215 GB in FP64, do not fit the device at once); each batch's run is one persistent
    integration launch over its (star, phase, tile) items, timed as issued and as a CUDA
    graph replay, with the launch shape of the tuned cache.  Beside it: the same stars as
    queued single-star calls (soapgb_disk_maps, soapgb_quiet_disk x2,
    soapgb_phase_pipeline per star, device buffers)."""
    import ctypes
    import torch
    from soap_gpu_gb300 import autotune, synth
    from soap_gpu_gb300._lib import Activity, Star
    from soap_gpu_gb300.api import Batch
    stars = synth.make_batch(n_star, seed=3)
    act = Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, 0)
    lb = inp.lb
    sts = [Star(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, (ctypes.c_double * 4)(*lb))
           for c in stars]
    n_eff = case.n_eff
    total_phases = sum(c.n_phase for c in stars)
    mu_d = torch.as_tensor(inp.mu_boundary, device=dev)
    out_one = torch.empty((max(c.n_phase for c in stars), 3, n_eff), dtype=torch.float64, device=dev)

    def per_star():
        for c, st in zip(stars, sts):
            maps = ctx.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, mu_d, lb)
            qn = ctx.quiet_disk("fast32", wave_d, cubes_d["q_norm"], n_eff, maps, c.grid, case.step)
            qs = ctx.quiet_disk("fast32", wave_d, cubes_d["q_sed"], n_eff, maps, c.grid, case.step)
            ctx.phase_pipeline("fast32", wave_d, n_eff, st, maps, cubes_d, case.step, act, c.phases,
                               [c.regions for _ in c.phases], qs, qn, case.sigma_v, conv_step=case.step,
                               out=out_one[:c.n_phase])

    ms_single = timed_steps(per_star, 1, stream)
    del out_one
    torch.cuda.empty_cache()
    ms_run = ms_graph = create_s = 0.0
    shapes, items, dev_bytes = [], 0, 0
    for k in range(0, n_star, per_batch):
        sub = stars[k:k + per_batch]
        t0 = time.perf_counter()
        b = Batch(ctx, wave_d, n_eff, cubes_d, inp.mu_boundary, case.step, act, case.sigma_v,
                  sts[k:k + per_batch], [c.phases for c in sub], [[c.regions for _ in c.phases] for c in sub],
                  conv_step=case.step)
        create_s += time.perf_counter() - t0
        grids = [c.grid for c in sub]
        shape = autotune.shape_for(b, grids)
        if shape is not None:
            b.tune(*shape)
        shapes.append({"class": autotune.key_of(b, grids), "shape": shape})
        items += b.items
        dev_bytes = max(dev_bytes, b.device_bytes)
        out = torch.empty((b.total_phases, 3, n_eff), dtype=torch.float64, device=dev)
        ms_run += timed_steps(lambda: b.run(out), 1, stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            b.run(out)
        ms_graph += timed_steps(g.replay, 1, stream)
        del g
        b.close()
        del out
        torch.cuda.empty_cache()
    return {"stars": n_star, "phases": total_phases, "visible_phases": items,
            "value": round(total_phases / (ms_graph / 1e3), 2), "unit": UNIT,
            "ms_graph_replay": round(ms_graph, 2), "ms_run": round(ms_run, 2),
            "value_run": round(total_phases / (ms_run / 1e3), 2),
            "single_star_calls": {"ms": round(ms_single, 2), "value": round(total_phases / (ms_single / 1e3), 2)},
            "speedup_vs_single_star_calls": round(ms_single / ms_graph, 3),
            "batches": "%d batches of up to %d stars, one persistent integration launch each" %
                       ((n_star + per_batch - 1) // per_batch, per_batch),
            "create_s": round(create_s, 3), "device_bytes_max": int(dev_bytes), "tuned_shapes": shapes,
            "what": "every stage per star: disk maps, 2 quiet spectra, lists, plans, integration, convolution, "
                    "normalisation; FP32 form; inputs resident"}


def ref_cuda_record(n_phase):
    """The reference's own CUDA programs (patched for determinism) on the 300x300 /
    310,000-px star, as run_all_SOAP.py runs them (one process per stage, float64 files
    between stages), from the committed record of oracle/ref_run.py."""
    p = os.path.join(ROOT, "oracle", "ref_cuda_record.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        rec = json.load(f)
    c1 = rec.get("case1", {})
    t = c1.get("patched", {}).get("times_s", {})
    if not t:
        return None
    ph = c1.get("phases", 10)
    per = (t.get("integration", 0.0) + t.get("resolution", 0.0)) / ph
    return {"value": round(1.0 / per, 3) if per > 0 else None, "unit": UNIT, "phases": ph,
            "integration_s": t.get("integration"), "resolution_s": t.get("resolution"),
            "includes": "process start, file reads and writes of each stage, as run_all_SOAP.py runs them",
            "source": "oracle/ref_cuda_record.json (" + rec.get("command", "python -m oracle.ref_run") + ")"}


def adjoint_timing(ctx, dev, reps=3):
    """Forward and forward + adjoint of the differentiable integration (PLAIN64,
    soap_gpu_gb300.differentiable) on one star of the differentiable-form shape: 200x200
    grid, 100,000 px, 3 regions, 5 phases over one rotation (of its 50); CUDA events,
    inputs resident."""
    import dataclasses
    import torch
    from soap_gpu_gb300 import synth
    from soap_gpu_gb300.differentiable import (IntegrationSetup, ResolutionSetup, deficit_spectra,
                                               lower_resolution)
    from soap_gpu_gb300._lib import Activity
    case = synth.small_case(seed=4, grid=200, n=100000, n_phase=5, n_mu=10)
    case = dataclasses.replace(case, regions=np.array([[20.0, 180.0, 0.1, 0.0], [-15.0, 200.0, 0.1732, 1.0],
                                                       [35.0, 160.0, 0.1, 1.0]]), rot_step=0.2)
    inp = synth.generate(case)
    n_eff = (case.n // 512) * 512
    setup = IntegrationSetup.build(ctx, inp.wave, n_eff, case.grid, case.period, case.w_ratio, case.incl,
                                   case.radius_km, inp.mu_boundary, inp.lb, case.phases,
                                   [case.regions for _ in case.phases],
                                   Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, 0), case.step,
                                   device=dev)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    cubes = [T(inp.q_norm), T(inp.q_sed), T(inp.spot_norm), T(inp.fac_norm), T(inp.spot_sed[0]), T(inp.fac_sed[0])]
    u = T([case.u1, case.u2, case.vsini])
    W = torch.ones((case.n_phase, 3, case.n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def fwd():
        with torch.no_grad():
            deficit_spectra(u, *cubes, setup)

    def fwd_bwd():
        ug = u.clone().requires_grad_(True)
        cg = [c.clone().requires_grad_(True) for c in cubes]
        (deficit_spectra(ug, *cg, setup) * W).sum().backward()

    # the chain on through the resolution step: low-resolution spectra of quiet - flux deficit
    maps = setup.maps(case.u1, case.u2, case.vsini)
    base = ctx.quiet_disk("plain64", setup.wave, cubes[1], n_eff, maps, case.grid, case.step).reshape(-1)
    rs = ResolutionSetup(ctx, setup.wave, n_eff, float(case.sigma_v))
    W2 = torch.ones((case.n_phase, n_eff), dtype=torch.float64, device=dev)

    def chain_fwd():
        with torch.no_grad():
            lower_resolution(deficit_spectra(u, *cubes, setup)[:, 0].contiguous(), base, rs)

    def chain_fwd_bwd():
        ug = u.clone().requires_grad_(True)
        cg = [c.clone().requires_grad_(True) for c in cubes]
        (lower_resolution(deficit_spectra(ug, *cg, setup)[:, 0].contiguous(), base, rs) * W2).sum().backward()

    f_ms, fb_ms = timed(fwd), timed(fwd_bwd)
    cf_ms, cfb_ms = timed(chain_fwd), timed(chain_fwd_bwd)
    return {"case": "200x200 grid, 100,000 px, 10 mu bins, 3 regions, 5 phases over one rotation, PLAIN64; "
                    "gradients w.r.t. u1, u2, vsini, 4 seed cubes, 2 continuum rows",
            "forward_ms": round(f_ms, 3), "forward_adjoint_ms": round(fb_ms, 3), "ratio": round(fb_ms / f_ms, 2),
            "with_resolution": {"case": "the same, then the resolution step (Gaussian convolution, min/max "
                                        "normalisation) of the quiet spectrum - flux deficit of each phase",
                                "forward_ms": round(cf_ms, 3), "forward_adjoint_ms": round(cfb_ms, 3),
                                "ratio": round(cfb_ms / cf_ms, 2)}}


def accuracy(ctx, case, inp, out_d, ref_d):
    """Error of a form's normalised spectra (out_d) against the plain FP64 form's
    (ref_d, the reference's arithmetic) on the same step: max relative flux error and
    the RV / BIS / FWHM differences of the CCF Gaussian fits, in cm/s."""
    import torch
    from soap_gpu_gb300 import rv
    n_eff = case.n_eff
    torch.cuda.synchronize()
    o, r = out_d.cpu().numpy(), ref_d.cpu().numpy()
    scale = np.max(np.abs(r), axis=2, keepdims=True)
    flux_err = float(np.max(np.abs(o - r) / scale))
    wave = inp.wave[:n_eff]
    series_o = rv.rv_series(ctx, case, wave, o, inp.mask_wave, inp.mask_weight)
    series_r = rv.rv_series(ctx, case, wave, r, inp.mask_wave, inp.mask_weight)
    d = {k: float(np.max(np.abs(series_o[k] - series_r[k])) * 100.0) for k in ("rv", "span", "fwhm")}
    return {"against": "plain64", "flux_rel_max": flux_err, "rv_cms_max": d["rv"], "bis_span_cms_max": d["span"],
            "fwhm_cms_max": d["fwhm"], "rv_range_ms": float(np.ptp(series_r["rv"]))}


def timed_steps(fn, steps, stream):
    """ms per call of fn over `steps` calls, CUDA events on `stream` (one warm-up call)."""
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def diff_batch_timing(ctx, dev, stream, n_star=8, chunk=10):
    """The differentiable form on its own shape: stars of a 200x200 grid, 100,000 px, 10 mu
    bins and 3 regions (random positions, 1-2 % of the hemisphere, spot or facula) over 50
    phases of one rotation, vsini 1-4 km/s, inclination 60-90 deg.  Per star: both quiet
    spectra, the deficit spectra of every phase, their resolution step, mask CCF and
    Gaussian + bisector fit, for the three types; loss = a fixed combination of the RV,
    FWHM and span series.  Forward alone (no gradient kept) against forward + every
    adjoint (gradients w.r.t. u1, u2, vsini, inclination, the spot and facula contrasts
    and the four seed cubes), phases checkpointed in chunks of `chunk`.  The stars are
    independent, so the cost is the per-star cost times the stars; `n_star` of the 64 of
    the shape are timed, and the per-star figures scale to 64."""
    import dataclasses
    import torch
    from soap_gpu_gb300 import synth, rv
    from soap_gpu_gb300._lib import Activity
    from soap_gpu_gb300.differentiable import (CcfSetup, IntegrationSetup, ResolutionSetup, CUBE_KEYS,
                                               rv_series_checkpointed)
    case = synth.make_case(4)
    inp = synth.generate(case)
    n_eff = case.n_eff
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    cubes = {k: T(v) for k, v in zip(CUBE_KEYS, (inp.q_norm, inp.q_sed, inp.spot_norm, inp.fac_norm,
                                                 inp.spot_sed[0], inp.fac_sed[0]))}
    wt = rv.trim(inp.wave[:n_eff])
    lw, lwt = rv.select_lines(wt, inp.mask_wave, inp.mask_weight)
    cs = CcfSetup(ctx, T(case.velocities), T(lw), T(lwt), T(wt), float(case.step),
                  mask_step=float(case.step), index_old=int(rv.WAVE_EXTEND / case.step))
    rng = np.random.default_rng(44)
    stars = []
    for k in range(n_star):
        reg = np.column_stack([rng.uniform(-50, 50, 3), rng.uniform(0, 360, 3), np.sqrt(rng.uniform(0.01, 0.02, 3)),
                               rng.integers(0, 2, 3).astype(float)])
        stars.append(dataclasses.replace(case, regions=reg, vsini=float(rng.uniform(1.0, 4.0)),
                                         incl=float(rng.uniform(60.0, 90.0)), u1=float(rng.uniform(0.25, 0.35)),
                                         u2=float(rng.uniform(0.3, 0.4))))
    act = Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, 0)
    setups = [IntegrationSetup.build(ctx, inp.wave, n_eff, c.grid, c.period, c.w_ratio, c.incl, c.radius_km,
                                     inp.mu_boundary, inp.lb, c.phases, [c.regions for _ in c.phases], act, c.step,
                                     device=dev) for c in stars]
    rs = ResolutionSetup(ctx, setups[0].wave, n_eff, float(case.sigma_v), step_mult=case.step, step_exp=case.step)

    def one(c, setup, grad, recompute=True):
        star = T([c.u1, c.u2, c.vsini, c.incl])
        contrast = T([1.0, 1.0])
        cb = dict(cubes)
        if grad:
            star.requires_grad_(True)
            contrast.requires_grad_(True)
            cb = {k: v.clone().requires_grad_(True) for k, v in cubes.items()}
        cb2 = dict(cb)
        cb2["spot_sed"] = contrast[0] * cb["spot_sed"]
        cb2["fac_sed"] = contrast[1] * cb["fac_sed"]
        out = rv_series_checkpointed(star, cb2, setup, rs, cs, chunk=chunk, kind=(0, 1, 2), recompute=recompute)
        loss = sum((o["rv"] + 0.1 * o["fwhm"] + o["span"]).sum() for o in out.values())
        if grad:
            loss.backward()
        return loss

    def fwd():
        with torch.no_grad():
            for c, s in zip(stars, setups):
                one(c, s, False)

    def fwd_bwd():
        for c, s in zip(stars, setups):
            one(c, s, True, recompute=False)

    def fwd_bwd_ckpt():
        for c, s in zip(stars, setups):
            one(c, s, True)

    f_ms = timed_steps(fwd, 1, stream)
    fb_ms = timed_steps(fwd_bwd, 1, stream)
    fbc_ms = timed_steps(fwd_bwd_ckpt, 1, stream)
    return {"case": "%d stars (of 64) x 50 phases, 200x200 grid, 100,000 px, 10 mu bins, 3 regions each, "
                    "PLAIN64; both quiet spectra, deficits, resolution, CCF, Gaussian + bisector fit of 3 types; "
                    "gradients w.r.t. u1, u2, vsini, inclination, 2 contrasts, 4 seed cubes; phases in chunks "
                    "of %d" % (n_star, chunk),
            "stars_timed": n_star, "forward_ms": round(f_ms, 1), "forward_adjoint_ms": round(fb_ms, 1),
            "ratio": round(fb_ms / f_ms, 2),
            "checkpointed": {"forward_adjoint_ms": round(fbc_ms, 1), "ratio": round(fbc_ms / f_ms, 2),
                             "what": "the same with each chunk's forward recomputed in the backward"},
            "forward_ms_per_star": round(f_ms / n_star, 1),
            "forward_adjoint_ms_per_star": round(fb_ms / n_star, 1),
            "forward_adjoint_s_for_64_stars": round(fb_ms / n_star * 64 / 1e3, 1)}


def ccf_fit_stage(ctx, case, inp, out_d, quiet_low_d, stream, reps=5):
    """The CCF + fit stage of one step (run_all_SOAP.py:256-412, timed there as "RV
    Calculation time"): the 300 phase spectra and the 3 quiet ones, trimmed, through the
    mask CCF (normalised, apodised) and the batched Gaussian + bisector fit, inputs
    resident.  One RV series is the n_phase + 1 spectra of one type, so a step gives 3."""
    import torch
    from soap_gpu_gb300 import rv
    dev = out_d.device
    n_eff = case.n_eff
    wave_trim = rv.trim(inp.wave[:n_eff])
    lw, lwt = rv.select_lines(wave_trim, inp.mask_wave, inp.mask_weight)
    wt_d = torch.as_tensor(wave_trim, device=dev)
    vel_d = torch.as_tensor(case.velocities, dtype=torch.float64, device=dev)
    lw_d, lwt_d = torch.as_tensor(lw, device=dev), torch.as_tensor(lwt, device=dev)
    n_spec = out_d.shape[0] * 3 + 3
    no_points = int(rv.WAVE_EXTEND / case.step)

    def stage():
        spectra = torch.cat([rv.trim(out_d).reshape(-1, wave_trim.size), rv.trim(quiet_low_d)], dim=0)
        ccf = ctx.ccf("plain64", vel_d, lw_d, lwt_d, wt_d, case.step, spectra, normalise=True,
                      wave_extend=rv.WAVE_EXTEND, mask_step=case.step, index_old=no_points)
        return ctx.gauss_bis(vel_d, ccf)

    ms = timed_steps(stage, reps, stream)
    res = stage()
    torch.cuda.synchronize()
    ok = bool((res["iters"] >= 0).all())
    return {"value": round(3 / (ms / 1e3), 2), "unit": "RV-series/s", "ms_per_step": round(ms, 3),
            "spectra_per_step": int(n_spec), "spectra_per_s": round(n_spec / (ms / 1e3), 1),
            "mask_lines": int(lw.size), "velocities": int(len(case.velocities)), "fits_converged": ok,
            "what": "trim + mask CCF (FP64 sums, normalised, apodised) + Gaussian/bisector fit of the %d spectra of "
                    "one step (3 RV series of %d spectra), inputs resident" % (n_spec, n_spec // 3)}


def ccf_fit_cpu(case, inp, out_np, sample=6):
    """The reference's CPU form of the same stage on a sample of spectra: the dense mask
    dot of CCF_func.py (oracle C) and the Gaussian + bisector fit of BIS_FIT2 (oracle C
    restatement), one host thread per spectrum as the reference spawns them."""
    import oracle
    from soap_gpu_gb300 import rv
    n_eff = case.n_eff
    wt = rv.trim(inp.wave[:n_eff])
    lw, lwt = rv.select_lines(wt, inp.mask_wave, inp.mask_weight)
    t0 = time.perf_counter()
    M = oracle.ccf_mask(case.velocities, lw, lwt, wt, case.step, mask_step=case.step,
                        index_old=int(rv.WAVE_EXTEND / case.step))
    t_mask = time.perf_counter() - t0
    rows = out_np.reshape(-1, n_eff)[:sample]
    t0 = time.perf_counter()
    for r in rows:
        oracle.gauss_bis(case.velocities, oracle.ccf_normalise(oracle.ccf(M, rv.trim(r))))
    dt = (time.perf_counter() - t0) / len(rows)
    per_series = (out_np.shape[0] + 1) * dt
    return {"value": round(1.0 / per_series, 4), "unit": "RV-series/s", "s_per_spectrum": round(dt, 4),
            "mask_build_s": round(t_mask, 3), "cores": 1, "kind": "port",
            "sample": "%d spectra: dense mask dot (CCF_func.py calculate_CCF_2) + Gaussian/bisector fit "
                      "(BIS_FIT2), oracle C; the mask is built once" % len(rows)}


def cpu_baseline(case, inp, sample_phases=1):
    """The reference path's CPU restatement (oracle, OpenMP) on a bounded sample:
    `sample_phases` phases of the same workload, integration + convolution."""
    import oracle
    nth = oracle.num_threads()
    n_eff = case.n_eff
    maps = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                            inp.mu_boundary, inp.lb)
    # the quiet spectra only scale the normalisation; a coarse-grid disk sum stands in
    qmaps = oracle.disk_maps(40, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                             inp.mu_boundary, inp.lb)
    q_norm = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, qmaps, 40, case.step)
    q_sed = oracle.quiet_disk(inp.wave, inp.q_sed, n_eff, qmaps, 40, case.step)
    ph = case.phases[len(case.phases) // 2: len(case.phases) // 2 + sample_phases]
    t0 = time.perf_counter()
    for p in ph:
        temp, bi = oracle.phase_maps(case.grid, case.nrho, case.incl, p, case.regions, case.t_star, case.t_diff_spot,
                                     case.t_diff_fac)
        f, b, t = oracle.phase_integrate(inp.wave, n_eff, case.grid, temp, bi, maps, inp.q_norm, inp.q_sed,
                                         inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], case.step)
        for spec, base in ((t, q_sed), (f, q_sed), (b, q_norm)):
            oracle.lower_resolution(inp.wave, base - spec, n_eff, case.sigma_v, step_mult=case.step,
                                    step_exp=case.step)
    dt = time.perf_counter() - t0
    return {"value": round(len(ph) / dt, 4), "unit": UNIT, "cores": nth, "kind": "port",
            "sample": "%d phase(s) of the same workload (maps + integration + 3 convolutions), oracle C with "
                      "OpenMP over pixels" % len(ph), "seconds": round(dt, 3)}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------
def run_reference(args):
    ws, rk, lr = rank_info()
    if rk != 0:
        return None
    from soap_gpu_gb300 import synth
    import oracle
    case = synth.make_case(1)
    inp = synth.generate(case)
    n_eff = case.n_eff
    maps = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                            inp.mu_boundary, inp.lb)
    qmaps = oracle.disk_maps(40, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                             inp.mu_boundary, inp.lb)
    q_norm = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, qmaps, 40, case.step)
    q_sed = oracle.quiet_disk(inp.wave, inp.q_sed, n_eff, qmaps, 40, case.step)

    def step(p):
        temp, bi = oracle.phase_maps(case.grid, case.nrho, case.incl, p, case.regions, case.t_star,
                                     case.t_diff_spot, case.t_diff_fac)
        f, b, t = oracle.phase_integrate(inp.wave, n_eff, case.grid, temp, bi, maps, inp.q_norm, inp.q_sed,
                                         inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], case.step)
        for spec, base in ((t, q_sed), (f, q_sed), (b, q_norm)):
            oracle.lower_resolution(inp.wave, base - spec, n_eff, case.sigma_v, step_mult=case.step,
                                    step_exp=case.step)

    # steps walk the 100 phases with stride 37, so that a short run samples phases with
    # and without visible regions in proportion
    phases = case.phases
    pick = lambda k: phases[(37 * k) % len(phases)]
    for w in range(args.warmup):
        step(pick(w))
    t0 = time.perf_counter()
    for s in range(args.steps):
        step(pick(args.warmup + s))
    dt = time.perf_counter() - t0
    value = args.steps / dt
    nth = oracle.num_threads()
    return {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "300x300 grid, 310,000 px, facula + spot, one phase per step (a bounded sample "
                                   "of the 100-phase job)", "form": "reference CPU restatement"},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": "one phase per step: maps + integration + 3 convolutions"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def profile_stage(args):
    """One stage of the path run a few times on a small case, for ncu captures of its
    kernels (nothing is timed or printed but a one-line note).  Stages: ccf (mask CCF +
    Gaussian/bisector fit of 303 spectra of the 300x300 / 310,000-px step), bisector
    (bisector injection of one 20 x 310,000 cube), adjoint (forward + adjoint of the
    differentiable chain, 200x200 grid, 100,000 px, 5 phases), batch (the batched form on
    8 stars of grids 100-160 and 20-40 phases sharing the 310,000-px seeds), plain64 (the
    plain FP64 pipeline, 2 phases)."""
    import ctypes
    import torch
    from soap_gpu_gb300 import rv, synth
    from soap_gpu_gb300._lib import Activity, Star
    from soap_gpu_gb300.api import Batch, Context
    torch.cuda.set_device(0)
    dev = "cuda:0"
    case, inp, phases = make_workload(0, args.phases, args.phase0)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    act = Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, 0)
    ctx = Context(0)
    wave_d = T(inp.wave)
    cubes_d = dict(q_norm=T(inp.q_norm), q_sed=T(inp.q_sed), spot_norm=T(inp.spot_norm), fac_norm=T(inp.fac_norm),
                   spot_sed=T(inp.spot_sed[0]), fac_sed=T(inp.fac_sed[0]))
    n_eff = case.n_eff
    st = args.profile_stage
    if st in ("ccf", "plain64"):
        maps_d = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                               T(inp.mu_boundary), inp.lb)
        form = "fast32" if st == "ccf" else "plain64"
        qn = ctx.quiet_disk(form, wave_d, cubes_d["q_norm"], n_eff, maps_d, case.grid, case.step)
        qs = ctx.quiet_disk(form, wave_d, cubes_d["q_sed"], n_eff, maps_d, case.grid, case.step)
        ph = phases if st == "ccf" else phases[45:47]
        out = ctx.phase_pipeline(form, wave_d, n_eff, star_struct(case, inp.lb), maps_d, cubes_d, case.step, act, ph,
                                 [case.regions for _ in ph], qs, qn, case.sigma_v, conv_step=case.step)
        if st == "ccf":
            low = torch.stack([ctx.lower_resolution("fast32", wave_d, q, n_eff, case.sigma_v, step_mult=case.step,
                                                    step_exp=case.step)[0].reshape(-1) for q in (qs, qs, qn)])
            for _ in range(3):
                ccf_fit_stage(ctx, case, inp, out, low, torch.cuda.current_stream(), reps=1)
    elif st == "bisector":
        rng_b = np.random.default_rng(11)
        co = T(rng_b.uniform(-300.0, 300.0, (case.n_mu, 4)))
        for _ in range(3):
            ctx.bisector_inject(wave_d, T(inp.q_norm[0]), co)
    elif st == "adjoint":
        adjoint_timing(ctx, dev, reps=1)
    elif st == "batch":
        # a small batch (8 stars, grids 100-160, 20-40 phases: about 2 GB on the device)
        stars = synth.make_batch(8, seed=3, grid=(100, 160), n_phase=(20, 40))
        sts = [Star(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, (ctypes.c_double * 4)(*inp.lb))
               for c in stars]
        b = Batch(ctx, wave_d, n_eff, cubes_d, inp.mu_boundary, case.step, act, case.sigma_v, sts,
                  [c.phases for c in stars], [[c.regions for _ in c.phases] for c in stars], conv_step=case.step)
        for _ in range(2):
            b.run()
        b.close()
    torch.cuda.synchronize()
    ctx.close()
    return {"profile_stage": st, "done": True}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--form", default="fast32", choices=["fast32", "fast64", "plain64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batch", action="store_true", help="skip the 256-star batched form")
    ap.add_argument("--diff-stars", type=int, default=2,
                    help="stars of the differentiable shape (64 stars x 50 phases) to time; 0 skips it")
    ap.add_argument("--profile-only", action="store_true",
                    help="run only the warm-up and timed device steps (for ncu launch lists)")
    ap.add_argument("--phases", type=int, default=100, help="phases per step (100 is the benchmarked workload)")
    ap.add_argument("--phase0", type=int, default=0, help="index of the first phase (profiling subsets)")
    ap.add_argument("--profile-stage", default=None, choices=["ccf", "bisector", "adjoint", "batch", "plain64"],
                    help="run one stage a few times on a small case (for ncu captures)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "own":
        args.warmup = 3
    if args.profile_stage:
        print(json.dumps(profile_stage(args)))
        return
    res = run_reference(args) if args.impl == "reference" else run_own(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
