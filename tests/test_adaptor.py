"""The reference-side adaptor (hyperflow_gb300/adaptor/gpu_scheme.h: GpuScheme and
GpuForwardEuler behind the reference's Scheme / ODESolver interfaces) compiled and linked
against the reference's own headers and solver sources (`make -C oracle adaptor`), where the
reference tree is present.  The check program steps the reference's objects and the adaptor side
by side and compares the fields bit for bit when a GPU is visible; without one it reports the
missing device (exit 3), which still shows that the binding matches the reference's real
interfaces."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
LIB = os.path.join(ROOT, "hyperflow_gb300", "libhyperflow_gb300.so")


def test_adaptor_builds_against_the_reference_and_runs(tmp_path):
    if subprocess.run(["make", "-s", "-C", ORACLE, "has-ref"]).returncode != 0:
        pytest.skip("the reference tree is not on this machine")
    if not os.path.exists(LIB):
        pytest.skip("libhyperflow_gb300.so is not built")
    r = subprocess.run(["make", "-s", "-C", ORACLE, "adaptor"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    from hyperflow_gb300 import cases
    case = tmp_path / "case.json"
    case.write_text(json.dumps(cases.forward_facing_step_case(20, limiter="VanLeer")))
    run = subprocess.run([os.path.join(ORACLE, "_ref", "adaptor_check"), str(case), "6"],
                         capture_output=True, text=True, timeout=600)
    if run.returncode == 3:
        assert "reference objects built; no GPU context" in run.stdout
    else:
        assert run.returncode == 0 and " 0 differing values" in run.stdout, run.stdout + run.stderr


def test_uns_adaptor_builds_against_the_reference_and_runs(tmp_path):
    """The same for the unstructured adaptor (gpu_uns_scheme.h), on the 240-quad channel mesh
    read by both sides from one mesh file (the reference's loader, its own format)."""
    import numpy as np
    from conftest import GOLDEN
    if subprocess.run(["make", "-s", "-C", ORACLE, "has-ref"]).returncode != 0:
        pytest.skip("the reference tree is not on this machine")
    if not os.path.exists(LIB):
        pytest.skip("libhyperflow_gb300.so is not built")
    r = subprocess.run(["make", "-s", "-C", ORACLE, "adaptor"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    from hyperflow_gb300 import meshgen
    g = np.load(os.path.join(GOLDEN, "uns_quad_channel_240.npz"), allow_pickle=True)
    mesh = tmp_path / "channel.hmsh"
    mesh.write_text(meshgen.hmsh_text(g["verts"], g["codes"]))
    case = json.loads(str(g["case"]))
    case["mesh"]["type"] = "hyperflow_structured"
    case["mesh"]["file"] = str(mesh)
    path = tmp_path / "case.json"
    path.write_text(json.dumps(case))
    run = subprocess.run([os.path.join(ORACLE, "_ref", "adaptor_uns_check"), str(path), "8"],
                         capture_output=True, text=True, timeout=600)
    if run.returncode == 3:
        assert "reference objects built; no GPU context" in run.stdout
    else:
        assert run.returncode == 0 and " 0 differing values" in run.stdout, run.stdout + run.stderr
