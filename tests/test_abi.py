"""The C-ABI library loads without a GPU and exports every entry point the public
headers declare; host-side argument and case-file checks work with no device."""
import ctypes as C
import glob
import json
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(hf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "hf_create" in names and "hf_run" in names and len(names) >= 15


def test_library_exports_every_declared_symbol():
    from hyperflow_gb300 import _lib
    L = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from hyperflow_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), set(declared_symbols()) - set(_lib.SIGNATURES)


def _create(text):
    from hyperflow_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    raw = text.encode()
    st = L.hf_create(raw, len(raw), C.byref(h))
    msg = L.hf_last_error_message(h).decode() if h else ""
    if h:
        L.hf_destroy(h)
    return st, msg


def test_bad_json_is_a_parse_error():
    st, msg = _create("{ not json")
    assert st == 2


def test_missing_key_is_a_parse_error():
    from hyperflow_gb300 import cases
    c = cases.quadrant_case(16)
    del c["simulation"]["cfl"]
    st, msg = _create(json.dumps(c))
    assert st == 2 and "cfl" in msg


def test_unsupported_scheme_and_limiter():
    from hyperflow_gb300 import cases
    c = cases.quadrant_case(16)
    c["scheme"]["type"] = "WENO"
    assert _create(json.dumps(c))[0] == 3
    c = cases.quadrant_case(16, scheme="MUSCLHancock", limiter="Superbee")
    assert _create(json.dumps(c))[0] == 3


def test_status_strings():
    from hyperflow_gb300 import _lib
    L = _lib.lib()
    assert L.hf_status_string(0) == b"ok"
    assert L.hf_status_string(7) == b"no CUDA device"


def test_no_device_is_reported_not_faked():
    """With a valid case and no GPU visible, creation fails loudly (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from hyperflow_gb300 import cases
    st, _ = _create(json.dumps(cases.quadrant_case(16)))
    assert st == 7


def test_blocks_narrower_than_two_ghosts_are_refused():
    """hf_create refuses them before touching the GPU (no device needed)."""
    import ctypes as C
    import json
    from hyperflow_gb300 import cases
    from hyperflow_gb300._lib import lib
    L = lib()
    for scheme, nx, ny in (("Godunov", 1, 5), ("MUSCLHancock", 3, 8), ("MUSCLHancock", 8, 2)):
        raw = json.dumps(cases.quadrant_case(nx, ny=ny, scheme=scheme,
                                             limiter=None if scheme == "Godunov" else "MinBee")).encode()
        h = C.c_void_p()
        st = L.hf_create(raw, len(raw), C.byref(h))
        msg = L.hf_last_error_message(h).decode()
        if h:
            L.hf_destroy(h)
        assert st == 3 and "2*ghost" in msg
