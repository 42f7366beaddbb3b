"""The reference module's import name, served by the GPU library.

The reference's optimisation scripts start with ``import pysplishsplash as sph`` (the
pybind11 module built from pySPlisHSPlasH/main.cpp:47-76). This package answers that
import with the surface of ``difffr_gb300.pysplishsplash`` -- ``sph.Exec.SimulatorBase``,
``sph.GUI.Simulator_GUI_imgui``, ``sph.Simulation``, ``sph.TimeManager``,
``sph.Utilities.Timing`` and the objects they return -- so that those scripts drive the
CUDA implementation without edits. Put the repository root on ``sys.path`` (or install
it) to make the name importable.
"""
from difffr_gb300.pysplishsplash import *  # noqa: F401,F403
from difffr_gb300.pysplishsplash import (  # noqa: F401
    GUI, BoundaryModelAkinci2012, Exec, RigidBodyGradientManager, RigidBodyObject, Simulation,
    TimeManager, TimeStepDiffDFSPH, Utilities)
