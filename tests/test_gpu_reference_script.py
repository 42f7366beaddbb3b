"""The reference's own optimisation script, run unchanged against the GPU library.

experiments/rigid_body_trajectory_optimization/python/gradient-based-optimize.py is read
from a DiffFR checkout (DIFFFR_REFERENCE, else ``reference`` beside this repository; the
test skips without one) and executed as ``__main__`` with its own command line. Its
``import pysplishsplash as sph`` is answered by this repository's ``pysplishsplash``
package. Its ``import quaternion`` (numpy-quaternion; the script imports it and never uses
it) is answered by an empty module where the package is not installed.

The scene is a small synthetic one in the reference's scene-JSON format: a fluid block in
a closed box and a dynamic sphere released into it, a trajectory of 12 steps. The script
runs the bottle-flip task (position and rotation losses, gradients from
get_grad_x_to_v0 / get_grad_quaternion_to_omega0) for two optimisation iterations and
then quits by itself (``--maxIter 1``).
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


def _script():
    ref = os.environ.get("DIFFFR_REFERENCE_SCRIPTS") or reference_root()
    if ref is None:
        return None
    p = os.path.join(ref, *SCRIPT)
    return p if os.path.exists(p) else None


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
    monkeypatch.setattr(sys, "argv", [script, "--scene", str(f), "--no-gui", "--no-initial-pause",
                                      "--taskType", "bottle-flip", "--maxIter", "1", "--lr-v", "0.1",
                                      "--lr-omega", "0.1", "--output-dir", str(tmp_path)])
    with pytest.raises(SystemExit):
        runpy.run_path(script, run_name="__main__")
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
    import pysplishsplash
    assert pysplishsplash.__file__.startswith(root)
