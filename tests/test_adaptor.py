"""The reference-side adaptors (hyperflow_gb300/adaptor/gpu_scheme.h: GpuScheme and
GpuForwardEuler behind the reference's Scheme / ODESolver interfaces; gpu_uns_scheme.h for the
unstructured solver) compiled and linked against the reference's own headers and solver sources
(`make -C oracle adaptor`).  The sources are the reference tree where it is present, else the
copy `make -C oracle stage` leaves in oracle/_ref/stage (git-ignored; it travels with the working
tree to the GPU host).

Two checks per solver:
* step by step: the reference's objects and the adaptor stepped side by side with the body of
  Simulation::solve, fields compared bit for bit;
* Simulation::solve itself: the reference's own, unmodified solve loop run to t_end twice -- with
  its own scheme and ODE solver, and with the adaptors in their place -- and every CSV frame it
  writes compared byte for byte.
Without a GPU the programs build the reference objects and report the missing device (exit 3),
which still shows the adaptors compile and link against the reference's real interfaces; the
`gpu`-marked tests require the comparisons to run and to find no difference."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
LIB = os.path.join(ROOT, "hyperflow_gb300", "libhyperflow_gb300.so")


def _build_or_skip():
    from oracle import make_args, reference_present
    if not reference_present():
        pytest.skip("neither the reference tree nor its staged copy (oracle/_ref/stage) is here")
    if not os.path.exists(LIB):
        pytest.skip("libhyperflow_gb300.so is not built")
    r = subprocess.run(["make", "-s", "-j4", "-C", ORACLE, *make_args(), "adaptor"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def _cart_case(tmp_path, t_end=None):
    from hyperflow_gb300 import cases
    case = cases.forward_facing_step_case(20, limiter="VanLeer")
    if t_end is not None:
        case["simulation"]["t_end"] = t_end
        case["simulation"]["animation"] = {"duration": 1.0, "fps": 10.0}
    path = tmp_path / "case.json"
    path.write_text(json.dumps(case))
    return path


def _uns_case(tmp_path, t_end=None):
    import numpy as np
    from conftest import GOLDEN
    from hyperflow_gb300 import meshgen
    g = np.load(os.path.join(GOLDEN, "uns_scramjet_reduced4.npz"), allow_pickle=True)
    mesh = tmp_path / "scramjet.hmsh"
    mesh.write_text(meshgen.hmsh_text(g["verts"], g["codes"]))
    case = json.loads(str(g["case"]))
    case["mesh"]["file"] = str(mesh)
    if t_end is not None:
        case["simulation"]["t_end"] = t_end
        case["simulation"]["animation"] = {"duration": 1.0, "fps": 8.0}
    path = tmp_path / "case.json"
    path.write_text(json.dumps(case))
    return path


def _run(prog, *args):
    return subprocess.run([os.path.join(ORACLE, "_ref", prog), *map(str, args)], capture_output=True,
                          text=True, timeout=900)


def _cpu_ok(run, verdict):
    if run.returncode == 3:
        assert "reference objects built; no GPU context" in run.stdout
    else:
        assert run.returncode == 0 and verdict in run.stdout + run.stderr, run.stdout[-2000:] + run.stderr


def test_adaptor_builds_against_the_reference_and_runs(tmp_path):
    _build_or_skip()
    _cpu_ok(_run("adaptor_check", _cart_case(tmp_path), 6), " 0 differing values")


def test_uns_adaptor_builds_against_the_reference_and_runs(tmp_path):
    """The unstructured adaptor on the reference's scramjet case (quartered cell counts), read by
    both sides from one mesh file (the reference's loader and format)."""
    _build_or_skip()
    _cpu_ok(_run("adaptor_uns_check", _uns_case(tmp_path), 8), " 0 differing values")


@pytest.mark.gpu
@pytest.mark.parametrize("prog,make_case,steps", [("adaptor_check", _cart_case, 25),
                                                  ("adaptor_uns_check", _uns_case, 40)])
def test_gpu_adaptor_steps_equal_reference(prog, make_case, steps, tmp_path):
    """Simulation::solve's step body, the reference's objects against the adaptor on the GPU:
    no differing value (cart: the 3-block forward-facing step, Van Leer; uns: the scramjet)."""
    _build_or_skip()
    run = _run(prog, make_case(tmp_path), steps)
    assert run.returncode == 0 and " 0 differing values" in run.stdout, run.stdout[-2000:] + run.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("prog,make_case,t_end", [("adaptor_check", _cart_case, 0.5),
                                                  ("adaptor_uns_check", _uns_case, 2e-4)])
def test_gpu_reference_simulation_solve_through_adaptor(prog, make_case, t_end, tmp_path):
    """The reference's own Simulation::solve, unmodified, with the adaptors as its scheme and ODE
    solver: every frame it writes equals, byte for byte, what it writes with its own scheme."""
    _build_or_skip()
    out = tmp_path / "solve"
    out.mkdir()
    run = _run(prog, make_case(tmp_path, t_end), 0, out)
    assert run.returncode == 0, run.stdout[-2000:] + run.stderr
    assert "differing frames" in run.stderr and " 0 differing frames" in run.stderr, run.stderr
    frames = int(run.stderr.split("Simulation::solve: ")[1].split(" frames")[0])
    assert frames >= 5
