"""The C-ABI library builds, loads, exports every entry point declared in
include/branson_gb300.h, and refuses to run without an sm_103 GPU (no CPU
fallback).  No compute call is made here."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^BGS_API\s+[\w\s\*]+?\b(bgs_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "bgs_replicated_transport" in names and "bgs_step" in names and len(names) >= 20


def test_library_exports_every_declared_symbol():
    from branson_gb300 import _lib
    lib = _lib.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) == bound


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from branson_gb300 import _lib
    lib = _lib.load()
    ctx = C.c_void_p()
    rc = lib.bgs_create(C.byref(ctx), 0, 16, None, 777, 100)
    assert rc == _lib.ERR_NO_DEVICE
    assert lib.bgs_status_string(rc) == b"no usable sm_103 device"


def test_bank_capacity_limit_is_checked_first():
    """Bank indices are 32-bit on the device: bgs_create rejects a capacity
    of 2^32 photons before it looks for a device."""
    from branson_gb300 import _lib
    lib = _lib.load()
    ctx = C.c_void_p()
    assert lib.bgs_create(C.byref(ctx), 0, 1 << 32, None, 777, 100) == _lib.ERR_INVALID
    assert not ctx.value


def test_engine_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from branson_gb300 import deck as D
    from branson_gb300.engine import ReplicatedIMC
    from branson_gb300._lib import BransonError
    with pytest.raises(BransonError):
        ReplicatedIMC(D.marshak_wave(photons=100))


def test_every_entry_point_names_what_it_replaces():
    """Each section of the C ABI header cites the upstream interface its entry
    points replace (file:line), or says that the reference has no counterpart."""
    lines = open(os.path.join(ROOT, "include", "branson_gb300.h")).read().splitlines()
    missing = []
    for i, line in enumerate(lines):
        m = re.match(r"^BGS_API\s+[\w\s\*]+?\b(bgs_\w+)\s*\(", line)
        if not m:
            continue
        j = i
        while j > 0 and not lines[j].startswith("/* ----"):
            j -= 1
        section = "\n".join(lines[j:i + 1])
        if not (re.search(r"\w+\.(h|in):\d+", section) or "counterpart" in section):
            missing.append(m.group(1))
    assert not missing, missing
