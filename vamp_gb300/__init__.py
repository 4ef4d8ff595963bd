"""vamp_gb300: VAMP's collision-checking hot path on one GB300 (sm_103a).

The Python surface mirrors the reference's bindings (src/impl/vamp/bindings/robot_helper.hh and
environment.cc): an `Environment` built from primitives, and one object per robot (`panda`,
`ur5`, `fetch`, `baxter`) with `validate`, `validate_motion`, `fk`, `min_max_radii`,
`dimension`, `resolution`, plus batched `validate_batch` / `validate_motion_batch`;
`filter_pointcloud` (environment.cc:167-197) on the GPU, `Attachment`, `HeightField`, each
robot's `eefk` and `validate_vector_batch` (planning/validate.hh:23-63); and, with
no counterpart in the reference, `autotune`, `Batch` (checks replayed as one CUDA graph) and
`CollisionPredictor` (the learned block ordering).

The CUDA library is loaded on first use of any of those names; if it has not been built the
access raises ImportError (there is no CPU fallback).  Submodules that do not need the GPU
(build, scenes, robots, robotgen, factory, roadmap) import without it.
"""
from __future__ import annotations

_API = {"Environment", "Robot", "VampError", "SQRT_X86", "SQRT_EXACT", "panda", "ur5", "fetch", "baxter", "ROBOTS",
        "autotune", "Batch", "CollisionPredictor", "SCHEDULES", "filter_pointcloud", "filter_pointcloud_device",
        "Attachment", "HeightField", "make_heightfield", "array_to_heightfield"}


def __getattr__(name):
    if name in _API:
        from . import api

        return getattr(api, name)
    raise AttributeError(name)


def __dir__():
    return sorted(_API)
