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


def test_block_count_limits():
    """No blocks, and more than the 16 a context holds, are refused before any device work."""
    from hyperflow_gb300 import cases
    c = cases.quadrant_case(16)
    c["mesh"]["blocks"] = []
    st, msg = _create(json.dumps(c))
    assert st == 3 and "between 1 and 16" in msg
    c = cases.quadrant_case(16)
    c["mesh"]["blocks"] = [json.loads(json.dumps(c["mesh"]["blocks"][0])) for _ in range(17)]
    st, msg = _create(json.dumps(c))
    assert st == 3 and "between 1 and 16" in msg


def test_cell_counts_must_be_whole_and_bounded():
    from hyperflow_gb300 import cases
    for nx in (16.5, -4, 3e9, float("inf")):
        c = cases.quadrant_case(16)
        c["mesh"]["blocks"][0]["x_cells"] = nx
        st, msg = _create(json.dumps(c).replace("Infinity", "1e400"))
        assert st in (2, 3), (nx, st, msg)
        if st == 3:
            assert "whole numbers" in msg


def test_boundary_errors():
    """An unknown boundary type, an Internal side naming a missing block, and an Internal side
    between blocks whose shared extents differ are refused with their reasons."""
    from hyperflow_gb300 import cases
    c = cases.quadrant_case(16)
    c["mesh"]["blocks"][0]["boundaries"]["left"] = {"type": "Periodic"}
    st, msg = _create(json.dumps(c))
    assert st == 3 and "Periodic" in msg
    c = cases.quadrant_case(16)
    for blk in (3, -1, 0.5, 1e12):
        c["mesh"]["blocks"][0]["boundaries"]["right"] = {"type": "Internal", "block": blk}
        st, msg = _create(json.dumps(c))
        assert st == 1 and "missing block" in msg, blk
    ffs = cases.forward_facing_step_case(cells_per_unit=20)
    blocks = ffs["mesh"]["blocks"]
    for b, blk in enumerate(blocks):
        for side, bc in blk["boundaries"].items():
            if bc["type"] == "Internal":
                other = blocks[bc["block"]]
                key = "x_cells" if side in ("bottom", "top") else "y_cells"
                other[key] = other[key] + 1            # the shared side no longer matches
                st, msg = _create(json.dumps(ffs))
                assert st == 3 and "unequal extent" in msg
                return
    pytest.fail("the forward-facing step has no Internal side")


def _uns_create(case, mesh: bytes):
    from hyperflow_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    raw = json.dumps(case).encode()
    st = L.hf_uns_create_mesh(raw, len(raw), mesh, len(mesh), C.byref(h))
    msg = L.hf_uns_last_error_message(h).decode() if h else ""
    if h:
        L.hf_uns_destroy(h)
    return st, msg


def _drop_last_code(text: bytes) -> bytes:
    """the text mesh with its last boundary code removed and the EDGES count lowered to match"""
    lines = text.rstrip(b"\n").split(b"\n")
    k = lines.index(b"EDGES")
    lines[k + 1] = str(int(lines[k + 1]) - 1).encode()
    return b"\n".join(lines[:-1]) + b"\n"


def _set_first_code(text: bytes, code: int) -> bytes:
    lines = text.rstrip(b"\n").split(b"\n")
    k = lines.index(b"EDGES")
    lines[k + 2] = str(code).encode()
    return b"\n".join(lines) + b"\n"


def _set_binary_code(data: bytes, ncells: int, code: int) -> bytes:
    import numpy as np
    off = 24 + 4 * ncells
    return data[:off] + np.array([code], "<i4").tobytes() + data[off + 4:]


def test_uns_mesh_parse_errors_need_no_device():
    """Malformed text and binary meshes are parse errors found before any device work; a valid
    mesh of either format gets as far as the device (no GPU here: HF_ERR_NO_DEVICE)."""
    import numpy as np
    import torch
    from hyperflow_gb300 import meshgen
    V, codes = meshgen.jittered_hole_mesh(300, seed=2)
    case = meshgen.channel_case("unused.hmsh")
    text = meshgen.hmsh_text(V, codes).encode()
    data = meshgen.hmshb_bytes(V, codes)
    lines = text.split(b"\n")
    bad = {
        "binary truncated": data[:-8],
        "binary header only": data[:20],
        "binary 5-vertex cell": data[:24] + np.array([5], "<i4").tobytes() + data[28:],
        "binary pair count": data[:16] + np.array([len(V) * 3 + 1], "<i8").tobytes() + data[24:],
        "text header": text.replace(b"CELLS", b"CELS", 1),
        "text cell count": text.replace(str(len(V)).encode(), str(len(V) + 1).encode(), 1),
        "text 2-vertex cell": b"\n".join(lines[:2] + [b"0.0 0.0 1.0 1.0"] + lines[3:]),
        # boundary codes: one per (cell, edge) pair, each -1, -2, -3 or a cell index
        "text fewer codes than pairs": _drop_last_code(text),
        "text code below -3": _set_first_code(text, -4),
        "text code past the cells": _set_first_code(text, len(V)),
        "binary code below -3": _set_binary_code(data, len(V), -4),
        "binary code past the cells": _set_binary_code(data, len(V), len(V)),
    }
    for what, mesh in bad.items():
        st, msg = _uns_create(case, mesh)
        assert st == 2 and "mesh" in msg, (what, st, msg)
    if not torch.cuda.is_available():
        # CRLF line endings and a missing final newline are read like the plain text
        for mesh in (text, data, text.replace(b"\n", b"\r\n"), text.rstrip(b"\n")):
            assert _uns_create(case, mesh)[0] == 7


def test_batch_manifest_cell_counts_are_checked_before_any_device_work():
    """Non-square, fractional, too small or too large batched cases are refused."""
    from hyperflow_gb300 import _lib, cases
    L = _lib.lib()
    for nx, ny in ((64, 65), (64.5, 64.5), (3, 3), (70000, 70000), (1e12, 1e12)):
        m = cases.batch_manifest(2, seed=0, side_min=64, side_max=80)
        blk = m["cases"][1]["mesh"]["blocks"][0]
        blk["x_cells"], blk["y_cells"] = nx, ny
        raw = json.dumps(m).encode()
        h = C.c_void_p()
        st = L.hf_batch_create(raw, len(raw), C.byref(h))
        msg = L.hf_batch_last_error_message(h).decode() if h else ""
        if h:
            L.hf_batch_destroy(h)
        assert st == 3 and "square" in msg, (nx, ny, st, msg)


def test_learned_solver_host_checks():
    """hf_lc_create refuses bad sizes before any device work; without a GPU it reports the missing
    device and still hands back a context whose setters check their arguments on the host: the
    inference path (0 separate kernels, 1 fused, 2 fused with the plain flux) and the fused
    kernel's CTAs per SM (0..4), the guard mode and bound."""
    import torch
    from hyperflow_gb300._lib import lib
    L = lib()
    h = C.c_void_p()
    assert L.hf_lc_create(3, 0.1, 1.4, 0.4, 0, C.byref(h)) == 1
    h = C.c_void_p()
    st = L.hf_lc_create(64, 1 / 64, 1.4, 0.4, 0, C.byref(h))
    assert st == (0 if torch.cuda.is_available() else 7) and h.value
    try:
        for mode, ctas in ((3, 0), (-1, 0), (1, 5), (1, -1)):
            assert L.hf_lc_set_fused(h, mode, ctas) == 1
        for mode, ctas in ((0, 0), (1, 4), (2, 1)):
            assert L.hf_lc_set_fused(h, mode, ctas) == 0
        assert L.hf_lc_set_guard_mode(h, 2) == 1 and L.hf_lc_set_guard_mode(h, 1) == 0
        assert L.hf_lc_set_bound(h, 0.0) == 1 and L.hf_lc_set_bound(h, 2.0) == 0
        assert L.hf_lc_set_fused(None, 1, 0) == 1
    finally:
        L.hf_lc_destroy(h)
