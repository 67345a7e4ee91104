"""ORACLE -- test infrastructure only.

Builds the reference's own CUDA programs (SOAP_initialize.cu, SOAP_integration.cu,
SOAP_integration_solar.cu, SOAP_resolution.cu) for sm_103a, in two variants, into
``oracle/_ref/`` (git-ignored; never part of the product):

* ``asis``    -- the unmodified sources;
* ``patched`` -- the same sources with the minimal edits that make their output
                 deterministic, so they can pin the GPU library's semantics:
  P1  fresh device and host buffers are zero (cudaMemset / calloc), and the
      per-cell interpolation buffers are cleared before every cell;
  P2  fast_interp_new never reads the shift of the source one past the processed
      range, and the mu-bin search never reads past the boundary array (the last
      bin is the default);
  P4  fast_interp_new writes every output pixel that its source interval owns
      ([ceil(x_i), ceil(x_{i+1})) -- no holes, no colliding writes);
  P6  the rim bounding box is reduced by one thread over all rim points instead
      of by every block reading the others' partial results;
  and the bounding box is clamped to the grid before the host scan.
  The -60000 max sentinel and the 0.005 A literals are left as written.

Sources are copied from the reference checkout (the ``SOAP_code`` directory named by
the argument or by ``SOAP_GPU_REF``) into ``oracle/_ref/src``; where no checkout is
given or present (the GPU host) the staged copies are compiled.  The binaries are the oracle's "reference" mode: only
tests and the parity scripts run them.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(REF_DIR, "src")
BIN = os.path.join(REF_DIR, "bin")
NAMES = ["SOAP_initialize", "SOAP_integration", "SOAP_integration_solar", "SOAP_resolution"]

# --- P4 + P2: the interval-owning interpolation (replaces fast_interp_new's body) --
INTERP_PATCHED = r'''__global__ void fast_interp_new(double *lambda, double *lambda_shift, double *spectrum, double *spec_grad, double *spectrum_out, double delta, double limb, double step_size, int offset){
    /* patched (P2, P4): source i owns the output pixels [ceil(x_i), ceil(x_{i+1})) */
    int index = blockIdx.x * blockDim.x + threadIdx.x;
    int n_eff = gridDim.x * blockDim.x;
    int index_offset = index + offset;
    double lambda0 = lambda[0];
    double c=299792458.;
    double beta = delta*1000./c;
    double fbeta = -1 * (1 - sqrt((1+beta)/(1-beta)));
    if (delta == 0.0){
        spectrum_out[index] = spectrum[index_offset]*limb;
        return;
    }
    if (index + 1 >= n_eff) return;
    int lo = (int) ceil(__dadd_rn(__dmul_rn((double)index, 1+fbeta), __ddiv_rn(__dmul_rn(fbeta, lambda0), step_size)));
    int hi = (int) ceil(__dadd_rn(__dmul_rn((double)(index+1), 1+fbeta), __ddiv_rn(__dmul_rn(fbeta, lambda0), step_size)));
    if (lo < 0) lo = 0;
    if (hi > n_eff) hi = n_eff;
    for (int j = lo; j < hi; j++)
        spectrum_out[j] = (spectrum[index_offset]+spec_grad[index_offset]/(lambda_shift[index+1] - lambda_shift[index])*(lambda[j] - lambda_shift[index]))*limb;
}
'''

# --- P6: one thread reduces all rim points -----------------------------------------
SPOT_AREA_P6 = r'''__global__ void spot_area_p6(double *xlylzl, int nrho, int grid, int *boundaries){
    /* patched (P6): sequential over the rim points */
    double grid_step = 2./grid;
    double miny=1, minz=1, maxy=-1, maxz=-1;
    int sum_on=0, sum_off=0;
    for (int jj=0; jj<nrho; jj++){
        if (xlylzl[3*jj] >= 0){
            sum_on++;
            if (xlylzl[3*jj+1]<miny) miny = xlylzl[3*jj+1];
            if (xlylzl[3*jj+2]<minz) minz = xlylzl[3*jj+2];
            if (xlylzl[3*jj+1]>maxy) maxy = xlylzl[3*jj+1];
            if (xlylzl[3*jj+2]>maxz) maxz = xlylzl[3*jj+2];
        } else sum_off++;
    }
    if (( sum_on >0)&&( sum_off >0)) {
        if (miny*maxy<0) { if (minz<0) minz=-1; else maxz=1; }
        if (minz*maxz<0) { if (miny<0) miny=-1; else maxy=1; }
    }
    boundaries[0] =(int) floor((1.+miny)/grid_step);
    boundaries[1] =(int) floor((1.+minz)/grid_step);
    boundaries[2] =(int) ceil((1.+maxy)/grid_step);
    boundaries[3] =(int) ceil((1.+maxz)/grid_step);
    boundaries[4] = sum_on == 0 ? 0 : 1;
}
'''


def _sub_kernel(text, name, replacement):
    m = re.search(r"__global__ void %s\(" % name, text)
    if not m:
        raise RuntimeError("patch anchor %s not found" % name)
    i = text.index("{", m.end())
    depth, j = 0, i
    while True:
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                break
        j += 1
    return text[:m.start()] + replacement + text[j + 1:]


def _must_replace(text, old, new, count=1):
    if text.count(old) < 1:
        raise RuntimeError("patch anchor not found: %r" % old[:60])
    return text.replace(old, new) if count == 0 else text.replace(old, new, count)


def patch(name, text):
    """Apply the oracle patch set to one reference source."""
    # P1: host buffers zeroed
    text = re.sub(r"\(double\*\)malloc\(\s*([^;]*?)\s*\*\s*sizeof\(double\)\s*\)", r"(double*)calloc(\1, sizeof(double))",
                  text)
    # P1: every device buffer zeroed right after allocation
    text = re.sub(r"(cudaMalloc\(\s*\(void\*\*\)&(\w+),([^;]*)\)\s*;)", r"\1 cudaMemset(\2, 0, \3);", text)
    if "fast_interp_new" in text:
        text = _sub_kernel(text, "fast_interp_new", INTERP_PATCHED)
    if name == "SOAP_initialize":
        # P2: mu-bin default is the last bin, the loop stays inside the boundary array
        text = _must_replace(text, "for (int id_mu = 0; id_mu<no_spec; id_mu++)",
                             "spec_idx = no_spec-1;\n                for (int id_mu = 0; id_mu<no_spec-1; id_mu++)")
        # P1: clear the per-cell buffer before each cell
        text = _must_replace(text, "fast_interp_new<<<no_block,no_thread>>>(dev_wav, dev_vrad, dev_spec, dev_grad, dev_spec_out,",
                             "cudaMemset(dev_spec_out, 0, vector_size*sizeof(double));\n                fast_interp_new<<<no_block,no_thread>>>(dev_wav, dev_vrad, dev_spec, dev_grad, dev_spec_out,")
    if name.startswith("SOAP_integration"):
        for buf in ("dev_spec_out,", "dev_spec_SED_out,", "dev_spec_out_spot,"):
            pat = re.compile(r"(\n\s*)(fast_interp_new<<<no_block,no_thread>>>\(dev_wav, dev_vrad, \w+, \w+, %s)" % re.escape(buf))
            if not pat.search(text):
                raise RuntimeError("patch anchor for %s not found" % buf)
            text = pat.sub(lambda m: "%scudaMemset(%s 0, vector_size*sizeof(double));%s%s" % (
                m.group(1), buf, m.group(1), m.group(2)), text)
        # P6: deterministic bounding box
        text = _must_replace(text, "__global__ void spot_init_gpu(", SPOT_AREA_P6 + "\n__global__ void spot_init_gpu(")
        text = _must_replace(text, "spot_area<<<nrho, 3>>>(xyz22, nrho, grid, boundaries, counton, countoff,maxminy_array,maxminz_array);",
                             "spot_area_p6<<<1, 1>>>(xyz22, nrho, grid, boundaries);")
        # the bounding box stays inside the grid
        text = _must_replace(text, "cudaMemcpy(boundaries_cpu, boundaries, 5*sizeof(int), cudaMemcpyDeviceToHost );",
                             "cudaMemcpy(boundaries_cpu, boundaries, 5*sizeof(int), cudaMemcpyDeviceToHost );\n"
                             "            for (int q = 0; q < 2; q++) if (boundaries_cpu[q] < 0) boundaries_cpu[q] = 0;\n"
                             "            for (int q = 2; q < 4; q++) if (boundaries_cpu[q] > grid) boundaries_cpu[q] = grid;")
    return text


def stage(checkout=None) -> bool:
    """Copy the reference sources next to the build (asis + patched)."""
    checkout = checkout or os.environ.get("SOAP_GPU_REF")
    if not checkout or not os.path.isdir(checkout):
        return os.path.isdir(os.path.join(SRC, "asis"))
    for variant in ("asis", "patched"):
        os.makedirs(os.path.join(SRC, variant), exist_ok=True)
    for name in NAMES:
        with open(os.path.join(checkout, name + ".cu")) as f:
            text = f.read()
        with open(os.path.join(SRC, "asis", name + ".cu"), "w") as f:
            f.write(text)
        with open(os.path.join(SRC, "patched", name + ".cu"), "w") as f:
            f.write(patch(name, text))
    return True


def build(quiet: bool = True, checkout=None) -> bool:
    """Stage (when the checkout is present) and compile both variants; returns
    False when neither the checkout nor staged sources exist."""
    if not stage(checkout):
        return False
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return False
    jobs = []
    for variant in ("asis", "patched"):
        os.makedirs(os.path.join(BIN, variant), exist_ok=True)
        for name in NAMES:
            src = os.path.join(SRC, variant, name + ".cu")
            exe = os.path.join(BIN, variant, name)
            if os.path.exists(exe) and os.path.getmtime(exe) >= os.path.getmtime(src):
                continue
            cmd = [nvcc, "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-ffp-contract=off",
                   "-w", "-o", exe, src]
            jobs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    ok = True
    for p in jobs:
        out, _ = p.communicate()
        if p.returncode != 0:
            ok = False
            if not quiet:
                print(out)
    return ok


if __name__ == "__main__":
    import sys
    print("built" if build(quiet=False, checkout=sys.argv[1] if len(sys.argv) > 1 else None)
          else "reference sources not available (pass the SOAP_code directory or set SOAP_GPU_REF)")
