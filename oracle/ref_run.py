"""ORACLE -- test infrastructure only.

Runs the reference's CUDA programs (oracle/_ref, both variants) and the drop-in
executables of this repository on the same synthetic inputs, through the same argv
contract run_all_SOAP.py uses (run_all_SOAP.py:160-250), and compares every file
they write.  Usage (on a GPU host, after ``__graft_entry__.build()``):

    python -m oracle.ref_run --case 0 --out ref_out/case0
    python -m oracle.ref_run --case 1 --phases 10 --rot-step 0.1 --out ref_out/case1

Writes ``summary.json`` under --out with the per-file differences and the wall time
of every stage of every implementation.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from soap_gpu_gb300 import config as cfgmod, synth  # noqa: E402


def prepare(case, root, n_phase=None, rot_step=None):
    """Synthetic inputs + the driver's map files (run_all_SOAP.py:160-220).  n_phase and
    rot_step override the case's (phases = arange(0, n_phase * rot_step, rot_step), as
    run_all_SOAP.py:191 forms them), so that a short run can still span the rotation."""
    if n_phase is not None:
        case.n_phase = n_phase
    if rot_step is not None:
        case.rot_step = rot_step
    inp = synth.generate(case)
    os.makedirs(root, exist_ok=True)
    cfg_path = synth.write_reference_layout(inp, root)
    return inp, cfg_path


def stage_argv(rc, root, exe_dir, solar=False):
    """The four command lines of run_all_SOAP.py:226-250 (paths relative to root)."""
    wave = np.fromfile(os.path.join(root, rc.input_dir, rc.wave_array_name))
    step_size = round(wave[3] - wave[2], 5)
    vector_size = int(wave.size)
    no_block = int(vector_size / rc.no_thread)
    n_mu = np.fromfile(os.path.join(root, rc.input_dir, rc.mu_array_name)).size + 1
    lbf = np.load(os.path.join(root, rc.input_dir, "Limb_brightening_info.npz"))
    lb = cfgmod.lb_params(rc.t_star, lbf["LB_G2"], lbf["LB_K0"], lbf["LB_M0"], lbf["Temp_array"])
    cp = rc.cube_paths
    out = rc.output_prefix + "/" + rc.file_prefix
    phase_txt = rc.output_prefix + "/" + rc.file_prefix + "_" + "phase_locator.txt"
    if rc.keyword == "real":
        # run_all_SOAP.py:148-157 reuses the phase locator already in place
        n_phase = int(np.atleast_1d(np.loadtxt(os.path.join(root, phase_txt))).size)
    else:
        n_phase = len(rc.phases)
    s = str
    init = lambda cube, pre: [os.path.join(exe_dir, "SOAP_initialize"), s(vector_size), s(rc.period),
                              s(rc.omega_ratio), s(rc.incl), s(rc.radius_km), s(rc.limb1), s(rc.limb2), s(rc.grid),
                              s(rc.inst_sigma), s(step_size), s(step_size), s(50.0), s(no_block), s(rc.no_thread),
                              cube, pre, s(n_mu), rc.input_dir + rc.mu_array_name, rc.input_dir + rc.wave_array_name,
                              s(lb[0]), s(lb[1]), s(lb[2]), s(lb[3])]
    integ = [os.path.join(exe_dir, "SOAP_integration_solar" if solar else "SOAP_integration"), s(rc.grid),
             s(rc.nrho), s(n_phase), s(rc.t_star), s(rc.t_diff_spot), s(rc.incl), s(rc.t_diff_fac), phase_txt,
             cp["fac_norm"], s(vector_size), rc.raw_dir, rc.maps_dir, s(no_block), s(rc.no_thread), cp["q_norm"],
             cp["spot_norm"], rc.file_prefix, s(step_size), s(n_mu), rc.input_dir + rc.wave_array_name, cp["q_sed"],
             cp["spot_sed"], cp["fac_sed"], rc.output_prefix + "/"]
    resol = [os.path.join(exe_dir, "SOAP_resolution"), s(n_phase), s(vector_size), s(rc.inst_sigma), rc.raw_dir,
             rc.final_spec_dir, s(no_block), s(rc.no_thread), rc.file_prefix, out]
    return [("initialize", init(cp["q_norm"], out)), ("initialize_sed", init(cp["q_sed"], out + "_SED")),
            ("integration", integ), ("resolution", resol)]


def write_maps(rc, root):
    """run_all_SOAP.py:160-220 (keyword != 'real')."""
    op = os.path.join(root, rc.output_prefix)
    if os.path.isdir(op):
        shutil.rmtree(op)
    for d in (rc.output_prefix, rc.maps_dir, rc.raw_dir, rc.final_spec_dir):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    phase_out = rc.phases
    np.savetxt(os.path.join(root, rc.output_prefix + "/" + rc.file_prefix + "_phase_locator.txt"), phase_out.T)
    info = np.zeros((phase_out.size, 2))
    for i in range(phase_out.size):
        cube = np.stack((rc.regions[:, 0], rc.regions[:, 1], rc.regions[:, 2], rc.regions[:, 3]), axis=1)
        np.savetxt(os.path.join(root, rc.maps_dir + "maps" + str(int(i)) + "_for_all.txt"), cube)
        info[i] = (i, rc.regions.shape[0])
    np.savetxt(os.path.join(root, rc.maps_dir + "final_info.txt"), info)


def run_impl(rc, root, exe_dir, env=None, stages=None, write=True):
    """Run the four stage programs in root; write=False keeps the phase locator and
    region files already there (the keyword 'real' layout, run_all_SOAP.py:148-157)."""
    if write:
        write_maps(rc, root)
    times = {}
    for name, argv in stage_argv(rc, root, exe_dir):
        if stages and name not in stages:
            continue
        t0 = time.perf_counter()
        p = subprocess.run(argv, cwd=root, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env,
                           timeout=3600)
        times[name] = time.perf_counter() - t0
        if p.returncode != 0:
            raise RuntimeError("%s failed (%d): %s" % (argv[0], p.returncode, p.stdout[-2000:]))
    return times


def collect(rc, root, n_eff):
    op = os.path.join(root, rc.output_prefix)
    files = {}
    for dirpath, _, names in os.walk(op):
        for nm in names:
            if nm.endswith(".bin"):
                rel = os.path.relpath(os.path.join(dirpath, nm), op)
                files[rel] = os.path.join(dirpath, nm)
    return files


def compare(a_files, b_files, n_eff):
    out = {}
    for rel in sorted(a_files):
        if rel not in b_files:
            out[rel] = "missing"
            continue
        dt = np.int32 if rel.endswith("region_map.bin") else np.float64
        a = np.fromfile(a_files[rel], dtype=dt)
        b = np.fromfile(b_files[rel], dtype=dt)
        if a.shape != b.shape:
            out[rel] = "shape %s vs %s" % (a.shape, b.shape)
            continue
        if dt == np.int32 or "map" in rel:
            nd = int(np.count_nonzero(a != b))
            d = {"exact": nd == 0, "n_diff": nd}
            if dt != np.int32 and nd:
                fin = np.isfinite(a) & np.isfinite(b)
                sc = max(float(np.max(np.abs(a[fin]))) if fin.any() else 0.0, 1e-300)
                d["max_rel"] = float(np.max(np.abs(a[fin] - b[fin]))) / sc if fin.any() else float("inf")
            out[rel] = d
            continue
        scale = max(float(np.max(np.abs(a))), 1e-300)
        full = float(np.max(np.abs(a - b)) / scale)
        inner = slice(210, a.size - 210) if a.size == n_eff else slice(0, a.size)
        out[rel] = {"full": full, "interior": float(np.max(np.abs(a[inner] - b[inner])) / scale)}
    return out


def summarise(diffs):
    agg = {}
    for rel, d in diffs.items():
        kind = rel.split("/")[-1]
        for tag in ("_Spec_tot", "_Spec_flux", "_Spec_bconv", "_lower_spec_tot", "_lower_spec_flux",
                    "_lower_spec_bconv", "_temp_map_", "_spot_binary_map_", "quiet_sun_spec", "quiet_sun_lower",
                    "mu_map", "delta_map", "limb_map", "LB_map", "region_map", "quiet_sun_wave"):
            if tag in kind:
                a = agg.setdefault(tag, {"files": 0})
                a["files"] += 1
                if not isinstance(d, dict):
                    a["error"] = d
                elif "interior" in d:
                    a["max_interior"] = max(a.get("max_interior", 0.0), d["interior"])
                    a["max_full"] = max(a.get("max_full", 0.0), d["full"])
                else:
                    a["exact"] = a.get("exact", True) and d["exact"]
                    a["n_diff"] = a.get("n_diff", 0) + d["n_diff"]
                    if "max_rel" in d:
                        a["max_rel"] = max(a.get("max_rel", 0.0), d["max_rel"])
                break
    return agg


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", type=int, default=0)
    ap.add_argument("--phases", type=int, default=None)
    ap.add_argument("--rot-step", type=float, default=None)
    ap.add_argument("--out", default="ref_out/run")
    ap.add_argument("--work", default="/tmp/soap_ref_run")
    ap.add_argument("--only-time", action="store_true")
    ap.add_argument("--impls", default="patched,asis,plain64,fast32")
    args = ap.parse_args()
    from oracle import ref_build
    from soap_gpu_gb300 import build as pkg_build
    case = synth.make_case(args.case)
    impls = args.impls.split(",")
    results = {"case": case.name, "timings": {}, "diff_vs_patched": {}}
    roots = {}
    for impl in impls:
        root = os.path.join(args.work, impl)
        inp, cfg_path = prepare(synth.make_case(args.case), root, args.phases, args.rot_step)
        rc = cfgmod.load_config(cfg_path)
        env = dict(os.environ)
        if impl in ("patched", "asis"):
            exe_dir = os.path.join(ref_build.BIN, impl)
        else:
            exe_dir = pkg_build.BINDIR
            env["SOAPGB_FORM"] = impl
        results["timings"][impl] = run_impl(rc, root, exe_dir, env=env)
        roots[impl] = (rc, root)
        print(impl, results["timings"][impl], flush=True)
    if not args.only_time and "patched" in roots:
        rc0, root0 = roots["patched"]
        base = collect(rc0, root0, case.n_eff)
        for impl in impls:
            if impl == "patched":
                continue
            rc1, root1 = roots[impl]
            d = compare(base, collect(rc1, root1, case.n_eff), case.n_eff)
            results["diff_vs_patched"][impl] = summarise(d)
    os.makedirs(args.out, exist_ok=True)
    with open(os.path.join(args.out, "summary.json"), "w") as f:
        json.dump(results, f, indent=1)
    print(json.dumps(results, indent=1))


if __name__ == "__main__":
    main()
