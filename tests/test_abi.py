"""The C-ABI library loads and exports every entry point declared in include/soapgb.h
(no compute calls: these tests run without a GPU)."""
import os
import re
import subprocess

import pytest

from soap_gpu_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "soapgb.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(soapgb_[a-z_0-9]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from soap_gpu_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("soapgb_ctx_create", "soapgb_quiet_disk", "soapgb_phase_integrate", "soapgb_lower_resolution",
              "soapgb_ccf", "soapgb_gauss_bis", "soapgb_phase_pipeline", "soapgb_disk_maps", "soapgb_phase_maps"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_python_binding_covers_every_symbol():
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_version_string(lib):
    assert lib.soapgb_version().decode().startswith("soapgb")


def test_null_context_is_rejected(lib):
    assert lib.soapgb_synchronize(None) == _lib.ERR_ARG
    assert lib.soapgb_last_error(None).decode() == "null context"


def test_dropin_executables_check_argv():
    """The argv checks run before any CUDA call: wrong argument counts fail loudly."""
    from soap_gpu_gb300 import build
    build.build()
    for name in build.TOOL_NAMES:
        exe = os.path.join(build.BINDIR, name)
        p = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        assert p.returncode == 1
        assert "expected" in p.stderr


def test_torch_operators_registered(lib):
    """The torch extension over the C ABI (torch.ops.soapgb.*) builds, loads and registers
    every operator (no compute calls)."""
    pytest.importorskip("torch")
    from soap_gpu_gb300 import build, torch_ops
    if not os.path.exists(torch_ops.PATH):
        build.build_torch_ops()
    o = torch_ops.load()
    for name in torch_ops.OPS:
        assert hasattr(o, name), name
