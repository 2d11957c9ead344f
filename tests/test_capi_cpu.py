"""Without a GPU: the C-ABI library exists and exports every entry point that
include/plum_gpu.h declares (no compute calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    out = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            out += re.findall(r"\b(plum_\w+)\s*\(", text)
    return sorted(set(out))


def test_library_exports_every_declared_symbol():
    import __graft_entry__
    import plum_gb300
    if not os.path.exists(plum_gb300.LIB_PATH):
        __graft_entry__.build()
    lib = ctypes.CDLL(plum_gb300.LIB_PATH)
    names = declared()
    assert "plum_ctx_create" in names and len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_product_does_not_reference_the_oracle():
    for dp, _, files in os.walk(os.path.join(ROOT, "plum_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cc", ".h", ".cuh")):
                text = open(os.path.join(dp, f)).read()
                assert "oracle" not in text.replace("the oracle", "").lower() or f == "systems.py", f


def test_compute_without_a_gpu_fails_loudly():
    """No CPU fallback: on a machine without a CUDA device, creating a
    context is an error (PLUM_ERR_CUDA), not a silent host computation."""
    import pytest
    import plum_gb300 as pg
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pg.PlumError) as ei:
        pg.System(os.path.join(ROOT, "tests", "golden", "bulk_small"))
    assert ei.value.code == 2
