"""GB300-native spectral-element guided-wave engine (flat shell, order 5).

Drop-in for the explicit central-difference loop of ma-shm's MATLAB solvers
(src/models/flat_shell/flat_shell_engine/main_flat_shell*.m).  The time loop
runs in ``libshmsem.so`` (CUDA, sm_103a) behind the C ABI in include/shmsem.h;
this package is the host side: meshes, materials, signals, plans and the
reference-shaped entry point ``main_flat_shell``.

The directory name contains a hyphen; import it through
``__graft_entry__.package()`` (it registers the module as ``mashm_gb300``).
"""
from . import build, element, materials, mesh, mesher, native, pzt, solver, wavefield, workloads  # noqa: F401
from .solver import Plan, RunConfig, Scenario, SolidPlan, SolidScenario, hanning_signal, main_flat_shell, main_flat_shell_multi_pzt_c, random_signal  # noqa: F401

__all__ = ["Plan", "RunConfig", "Scenario", "hanning_signal", "main_flat_shell", "main_flat_shell_multi_pzt_c", "build", "element", "materials", "workloads",
           "mesh", "native", "solver", "wavefield"]
