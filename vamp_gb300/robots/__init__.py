"""Robot models (JSON) extracted from the reference's URDFs and generated robot headers."""
from __future__ import annotations

import json
from functools import lru_cache
from pathlib import Path

HERE = Path(__file__).resolve().parent


@lru_cache(maxsize=None)
def model(name: str) -> dict:
    return json.loads((HERE / f"{name}.json").read_text())


def slot_count(name: str) -> int:
    """Fine spheres plus one coarse sphere per environment-checked link."""
    m = model(name)
    return len(m["fine_spheres"]) + len(m["env_checks"])
