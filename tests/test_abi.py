"""The C-ABI library loads and exports every symbol include/pxlflip.h declares (no GPU needed)."""
import os
import re
import subprocess

from pxlengine_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "pxlflip.h")).read()
    return sorted(set(re.findall(r"^PXF_API\s+[\w\s\*]+?\b(pxf_\w+)\(", text, re.M)))


def test_header_matches_binding(lib):
    syms = header_symbols()
    assert len(syms) >= 30
    assert sorted(L.EXPORTS) == syms


def test_library_exports_every_symbol(lib):
    for name in header_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pxf_\w+)", out))
    assert set(header_symbols()) <= exported
    # Nothing else leaks out of the library under the pxf_ prefix.
    assert exported == set(header_symbols())


def test_no_gpu_creation_fails_loudly(lib):
    import ctypes as C
    import pxlengine_gb300 as P
    try:
        import torch
        if torch.cuda.is_available():
            return
    except Exception:
        pass
    f = P.Fluid("w", [[0, 0, 0], [1, 1, 1]], [P.FluidBlock([0.2] * 3, [0.6] * 3)], resolution=16)
    out = C.c_void_p()
    rc = lib.pxf_create(C.byref(f.to_desc()), 0, 24.0, C.byref(out))
    assert rc == L.PXF_ECUDA and not out.value
    assert "CUDA" in lib.pxf_last_error(None).decode()
