"""Classification of verdict differences against the reference.

The kernels and the CPU oracle compute sphere centres with their own FP32 operation order; the
reference's compiled code uses another, so centres agree to a few 1e-7 m, not bit for bit.  A
verdict may therefore differ from the reference's only for a configuration within
CONTACT_TOL of contact (FP64 distance to contact).  Every difference is counted and checked
against that bound; anything else is an unexplained flip."""
from __future__ import annotations

import numpy as np

CONTACT_TOL = 1e-5  # metres


def motion_states(port_robot, a, b, resolution: int, lanes: int = 8) -> np.ndarray:
    """All states validate_motion would visit for one edge, as [states, dim] float32."""
    import ctypes

    lib = port_robot.port.lib
    n = lib.vgo_motion_block_count(port_robot.h, lanes, a.ctypes.data_as(ctypes.c_void_p),
                                   b.ctypes.data_as(ctypes.c_void_p), resolution)
    out = np.zeros((n, lanes, port_robot.dim), np.float32)
    lib.vgo_motion_blocks(port_robot.h, lanes, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                          resolution, out.ctypes.data_as(ctypes.c_void_p), n)
    return out.reshape(-1, port_robot.dim)


def classify_states(env, robot, q, mine, ref) -> dict:
    diff = np.nonzero(mine != ref)[0]
    dist = [abs(env.contact_distance(robot, q[i].astype(np.float64))) for i in diff]
    unexplained = [int(i) for i, d in zip(diff, dist) if d > CONTACT_TOL]
    return {"flips": len(diff), "unexplained": unexplained, "distances": dist}


def classify_edges(env, robot, a, b, resolution, mine, ref, lanes: int = 8) -> dict:
    diff = np.nonzero(mine != ref)[0]
    unexplained = []
    dists = []
    for i in diff:
        states = motion_states(robot, np.ascontiguousarray(a[i]), np.ascontiguousarray(b[i]), resolution, lanes)
        d = min(abs(env.contact_distance(robot, s.astype(np.float64))) for s in states)
        dists.append(d)
        if d > CONTACT_TOL:
            unexplained.append(int(i))
    return {"flips": len(diff), "unexplained": unexplained, "distances": dists}
