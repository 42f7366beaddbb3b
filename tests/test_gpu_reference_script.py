"""The reference's own optimisation scripts, run unchanged against the GPU library.

experiments/rigid_body_trajectory_optimization/python/gradient-based-optimize.py,
diff-rigid-contact-multi.py and experiments/bottle_flip_robot/python/bottle-flip-robot.py
are read from a DiffFR checkout (DIFFFR_REFERENCE_SCRIPTS, else
DIFFFR_REFERENCE, else ``reference`` beside this repository; the tests skip without one)
and executed as ``__main__`` with their own command lines. Its
``import pysplishsplash as sph`` is answered by this repository's ``pysplishsplash``
package. Its ``import quaternion`` (numpy-quaternion; the script imports it and never uses
it) is answered by an empty module where the package is not installed.

The scenes are small synthetic ones in the reference's scene-JSON format, trajectories of
12 steps. gradient-based-optimize.py runs the bottle-flip task (a fluid block in a closed
box and a dynamic sphere released into it; position and rotation losses, gradients from
get_grad_x_to_v0 / get_grad_quaternion_to_omega0); diff-rigid-contact-multi.py runs its
two-body task with the rigid contact solver and the gradient manager on (one sphere
strikes another; the gradient is the manager's cross-body block). Each runs two
optimisation iterations and then quits by itself (``--maxIter 1``).
"""
import json
import os
import re
import runpy
import sys
import types

import numpy as np
import pytest

from oracle import reference_root

pytestmark = pytest.mark.gpu

SCRIPT = ("experiments", "rigid_body_trajectory_optimization", "python", "gradient-based-optimize.py")
CONTACT_SCRIPT = ("experiments", "rigid_body_trajectory_optimization", "python", "diff-rigid-contact-multi.py")
ROBOT_SCRIPT = ("experiments", "bottle_flip_robot", "python", "bottle-flip-robot.py")


def _script(parts=SCRIPT):
    ref = os.environ.get("DIFFFR_REFERENCE_SCRIPTS") or reference_root()
    if ref is None:
        return None
    p = os.path.join(ref, *parts)
    return p if os.path.exists(p) else None


def _run_script(script, argv, tmp_path, monkeypatch, exits=True):
    """Runs a reference script as __main__ against this repository's pysplishsplash (exits:
    the script ends by quitting)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    monkeypatch.syspath_prepend(root)
    monkeypatch.syspath_prepend(os.path.dirname(script))
    try:
        import quaternion  # noqa: F401
    except ImportError:
        monkeypatch.setitem(sys.modules, "quaternion", types.ModuleType("quaternion"))
    for name in ("pysplishsplash", "utils"):
        monkeypatch.delitem(sys.modules, name, raising=False)
    monkeypatch.chdir(tmp_path)
    monkeypatch.setattr(sys, "argv", [script, *argv])
    if exits:
        with pytest.raises(SystemExit):
            runpy.run_path(script, run_name="__main__")
    else:
        runpy.run_path(script, run_name="__main__")
    import pysplishsplash
    assert pysplishsplash.__file__.startswith(root)


def test_gradient_based_optimize_runs_unchanged(gpu_lib, tmp_path, capsys, monkeypatch):
    script = _script()
    if script is None:
        pytest.skip("reference checkout not present")
    scene = {
        "Configuration": {"particleRadius": 0.025, "timeStepSize": 0.001, "targetTime": 0.012,
                          "maxIterations": 100, "maxError": 0.01, "maxErrorV": 0.1, "gradientMode": 1},
        "Materials": [{"id": "Fluid", "viscosity": 0.01}],
        "FluidBlocks": [{"start": [-0.3, 0.0, -0.3], "end": [0.3, 0.3, 0.3]}],
        "RigidBodies": [
            {"geometryFile": "UnitBox.obj", "scale": [1.0, 1.0, 1.0], "translation": [0.0, 0.45, 0.0],
             "isWall": True, "isDynamic": False},
            {"geometryFile": "sphere", "scale": [0.1, 0.1, 0.1], "translation": [0.0, 0.45, 0.0],
             "isDynamic": True, "density": 500, "initVelocity": [0.5, 0.0, 0.0],
             "initAngularVelocity": [0.0, 1.0, 0.0], "targetX": [0.2, 0.4, 0.0],
             "targetAngleInDegree": [0.0, 30.0, 0.0]},
        ],
    }
    f = tmp_path / "scene.json"
    f.write_text(json.dumps(scene))
    _run_script(script, ["--scene", str(f), "--no-gui", "--no-initial-pause", "--taskType", "bottle-flip",
                         "--maxIter", "1", "--lr-v", "0.1", "--lr-omega", "0.1", "--output-dir", str(tmp_path)],
                tmp_path, monkeypatch)
    out = capsys.readouterr().out
    losses = re.findall(r"===== iter (\d+), loss = \[tensor\(\[([-0-9.e+]+)\]", out)
    assert [int(i) for i, _ in losses] == [1, 2], out[-3000:]
    vals = np.array([float(v) for _, v in losses])
    assert np.all(np.isfinite(vals)) and np.all(vals > 0)
    # the script logged the gradient it used for both iterations
    grads = re.findall(r"grad_init_v_rb = \[([^\]]+)\]", out)
    assert len(grads) >= 2
    for g in grads:
        assert np.all(np.isfinite(np.array(g.split(), dtype=np.float64)))


def test_rigid_contact_multi_runs_unchanged(gpu_lib, tmp_path, capsys, monkeypatch):
    """experiments/rigid_body_trajectory_optimization/python/diff-rigid-contact-multi.py: the
    billiards-style task (the active sphere's initial velocity optimised so that the
    passive one it strikes reaches a target), with the rigid contact solver and the
    gradient manager on; the gradient is the manager's cross-body block
    get_grad_x_to_v0(passive, active). Two optimisation iterations on a small tank in which
    sphere 1 moves at 1 m/s towards sphere 2, 0.01 m away."""
    script = _script(CONTACT_SCRIPT)
    if script is None:
        pytest.skip("reference checkout not present")
    scene = {
        "Configuration": {"particleRadius": 0.025, "timeStepSize": 0.001, "targetTime": 0.012,
                          "maxIterations": 100, "maxError": 0.01, "maxErrorV": 0.1, "gradientMode": 1,
                          "useRigidContactSolver": True, "useRigidGradientManager": True},
        "Materials": [{"id": "Fluid", "viscosity": 0.01}],
        "FluidBlocks": [{"start": [-0.3, 0.0, -0.3], "end": [0.3, 0.2, 0.3]}],
        "RigidBodies": [
            {"geometryFile": "UnitBox.obj", "scale": [1.0, 1.0, 1.0], "translation": [0.0, 0.45, 0.0],
             "isWall": True, "isDynamic": False},
            {"geometryFile": "sphere", "scale": [0.1, 0.1, 0.1], "translation": [-0.105, 0.25, 0.0],
             "isDynamic": True, "density": 700, "initVelocity": [1.0, 0.0, 0.0],
             "initAngularVelocity": [0.0, 0.0, 0.0]},
            {"geometryFile": "sphere", "scale": [0.1, 0.1, 0.1], "translation": [0.105, 0.25, 0.0],
             "isDynamic": True, "density": 700, "initVelocity": [0.0, 0.0, 0.0],
             "initAngularVelocity": [0.0, 0.0, 0.0], "targetX": [0.3, 0.25, 0.0]},
        ],
    }
    f = tmp_path / "scene.json"
    f.write_text(json.dumps(scene))
    _run_script(script, ["--scene", str(f), "--no-gui", "--no-initial-pause", "--maxIter", "1",
                         "--act", "1", "--passive", "2", "--output-dir", str(tmp_path)], tmp_path, monkeypatch)
    out = capsys.readouterr().out
    losses = re.findall(r"===== iter (\d+), loss = \[tensor\(\[([-0-9.e+]+)\]", out)
    assert [int(i) for i, _ in losses] == [1, 2], out[-3000:]
    assert np.all(np.isfinite([float(v) for _, v in losses]))


def test_bottle_flip_robot_runs_unchanged(gpu_lib, tmp_path, capsys, monkeypatch):
    """experiments/bottle_flip_robot/python/bottle-flip-robot.py: a small policy network maps
    a target position to the bottle's initial velocities; each sample's trajectory runs
    through SimulatorBase.runNewTrajectory and the loss gradient comes from the boundary
    model's get_grad_x_to_v0 / get_grad_quaternion_to_omega0 blocks. One epoch over two
    training targets and one test target, batches of one. Its `from
    torch.utils.tensorboard.writer import SummaryWriter` is answered by a recorder of the
    logged scalars where tensorboard is not installed (the script only logs to it). The script
    moves its policy network to "cuda" when PyTorch sees a GPU but feeds it CPU tensors, so it
    only runs on the CPU-only PyTorch it was written with: PyTorch's GPU check answers False
    for it (the simulation itself still runs in the GPU library)."""
    script = _script(ROBOT_SCRIPT)
    if script is None:
        pytest.skip("reference checkout not present")
    scene = {
        "Configuration": {"particleRadius": 0.025, "timeStepSize": 0.001, "targetTime": 0.010,
                          "maxIterations": 100, "maxError": 0.01, "maxErrorV": 0.1, "gradientMode": 1},
        "Materials": [{"id": "Fluid", "viscosity": 0.01}],
        "FluidBlocks": [{"start": [-0.3, 0.0, -0.3], "end": [0.3, 0.3, 0.3]}],
        "RigidBodies": [
            {"geometryFile": "UnitBox.obj", "scale": [1.0, 1.0, 1.0], "translation": [0.0, 0.45, 0.0],
             "isWall": True, "isDynamic": False},
            {"geometryFile": "sphere", "scale": [0.1, 0.1, 0.1], "translation": [0.0, 0.45, 0.0],
             "isDynamic": True, "density": 500, "initVelocity": [0.5, 0.0, 0.0],
             "initAngularVelocity": [0.0, 1.0, 0.0], "targetX": [0.2, 0.4, 0.0],
             "targetAngleInDegree": [0.0, 30.0, 0.0]},
        ],
    }
    f = tmp_path / "scene.json"
    f.write_text(json.dumps(scene))
    (tmp_path / "saved_models").mkdir()
    scalars = []
    try:
        from torch.utils.tensorboard.writer import SummaryWriter  # noqa: F401
    except Exception:
        class _Writer:
            def add_scalar(self, tag, value, step):
                scalars.append((tag, float(value), int(step)))

            def close(self):
                pass
        mod = types.ModuleType("torch.utils.tensorboard.writer")
        mod.SummaryWriter = _Writer
        pkg = types.ModuleType("torch.utils.tensorboard")
        pkg.writer = mod
        monkeypatch.setitem(sys.modules, "torch.utils.tensorboard", pkg)
        monkeypatch.setitem(sys.modules, "torch.utils.tensorboard.writer", mod)
    import torch
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    np.random.seed(0)
    _run_script(script, ["--scene", str(f), "--no-gui", "--no-initial-pause", "--epoch", "1", "--batchsize", "1",
                         "--num-train", "2", "--num-test", "1", "--output-dir", str(tmp_path)],
                tmp_path, monkeypatch, exits=False)
    out = capsys.readouterr().out
    train = re.findall(r"loss: ([-0-9.e+]+)\[", out)
    assert len(train) == 2 and np.all(np.isfinite(np.array(train, dtype=np.float64))), out[-3000:]
    assert re.search(r"Avg loss: ([-0-9.e+]+)", out) and "Done!" in out
    assert sorted(os.listdir(tmp_path / "saved_models"))
