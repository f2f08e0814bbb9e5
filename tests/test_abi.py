"""The C-ABI library loads and exports every symbol include/pfstep.h declares;
the ctypes mirrors match the C struct sizes.  No GPU calls."""
import ctypes
import os
import re

import phasefield_gb300 as pf

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "pfstep.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, re.M)
    return sorted(set(n for n in names if n not in ("if", "while")))


def test_header_parses_expected_entry_points():
    names = declared_functions()
    for must in ("GPU_Init", "GPU_Diffusion_solver", "GPU_Cleanup", "pf_create", "pf_step", "pf_reduce",
                 "pf_upload_state", "pf_download_state", "pf_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = pf.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"not exported: {missing}"
    assert set(declared_functions()) <= set(pf.SYMBOLS), "ctypes table lacks a declared symbol"


def test_struct_sizes_match():
    out = (ctypes.c_longlong * 3)()
    assert pf.lib().pf_abi_sizes(out) == pf.PF_OK
    assert list(out) == [ctypes.sizeof(pf.PfModel), ctypes.sizeof(pf.PfStepParams), ctypes.sizeof(pf.PfInitSpec)]


def test_status_strings():
    L = pf.lib()
    assert L.pf_status_string(pf.PF_OK) == b"ok"
    assert L.pf_status_string(pf.PF_ERR_TIMEOUT) == b"device wait timed out"
