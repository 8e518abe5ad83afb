"""GB300 collision / distance / nearest-neighbour backend for multi-robot
multi-goal planners (drop-in beside the reference's abstract, rai, pinocchio
and mujoco environment backends).

The package directory name is not a Python identifier; import it with
``importlib.import_module("multirobot-pathplanning-benchmark_gb300")``.
"""
from .scenes import (  # noqa: F401
    AbstractScene,
    ArmScene,
    make_arm_scene,
    make_arm_workload,
    make_disc_scene,
    make_disc_workload,
    make_mobile_scene,
)

__all__ = [
    "AbstractScene",
    "ArmScene",
    "make_arm_scene",
    "make_arm_workload",
    "make_disc_scene",
    "make_disc_workload",
    "make_mobile_scene",
]


def __getattr__(name):
    # device-facing modules import torch and the CUDA library lazily
    if name in ("Gb300Scene", "binary_search_indices"):
        from . import collision

        return getattr(collision, name)
    if name in ("Gb300Configuration", "batch_config_dist", "batch_config_cost", "config_dist", "config_cost",
                "config_dist_matrix", "path_cost"):
        from . import configuration

        return getattr(configuration, name)
    if name in ("Gb300CollisionBackend", "Gb300AbstractEnvironment", "Gb300ArmEnvironment"):
        from . import env

        return getattr(env, name)
    raise AttributeError(name)
