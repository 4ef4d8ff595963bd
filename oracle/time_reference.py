"""Times the compiled reference (oracle/_ref: the reference's own validate_motion, its AVX2 build)
on the benchmark's edge workload, on this host's cores.

Test infrastructure: it runs only where the reference checkout and an x86-64 host are present
(not on the Arm GPU machine, which has neither).  bench.py reports its result beside the CPU baseline
it measures on the GPU machine, so that the basis of the GPU/CPU ratio is explicit.

    python oracle/time_reference.py [--reps 5]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or "unknown"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=5)
    a_ = ap.parse_args()
    from oracle.vgo import REF_LIB, Port, Reference
    from vamp_gb300 import scenes

    if not REF_LIB.exists():
        raise SystemExit("the reference oracle is not built (python -c 'import __graft_entry__ as g; g.build()')")
    rb = Port().robot("panda")
    scene, a, b = scenes.workload_config1(rb.s_m, rb.s_a)
    env = Reference().env(scene)
    env.validate_motions("panda", a[:2048], b[:2048], 32, 1)  # warm-up
    out = {"what": "compiled reference validate_motion (x86-64 AVX2 build, 8 lanes), 65,536 Panda edges at "
                   "resolution 32, config-1 scene", "host": cpu_model(), "when": time.strftime("%Y-%m-%d")}
    for threads in (1, os.cpu_count() or 1):
        ts = []
        for _ in range(a_.reps):
            t0 = time.perf_counter()
            env.validate_motions("panda", a, b, 32, threads)
            ts.append(time.perf_counter() - t0)
        out[f"threads_{threads}"] = {"threads": threads, "edges_per_s_best": len(a) / min(ts),
                                     "edges_per_s_median": len(a) / float(np.median(ts))}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
