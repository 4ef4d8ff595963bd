"""Straight-line forward-kinematics + collision-schedule generator.

Input: a robot model JSON (vamp_gb300/robots/<robot>.json, written by extract.py).
Output:
  * vamp_gb300/csrc/robots/<robot>.cuh  - CUDA device code for sm_103a: FP32 FK of every sphere and
    the robot's fkcc check schedule, written against a small context interface (see
    vamp_gb300/csrc/vg_check.cuh);
  * oracle/port/robots/<robot>.h        - C code for the CPU oracle: the same FP32 FK (bit-identical
    operation sequence), an FP64 FK for centre tolerances and distance-to-contact, and the check
    schedule as tables.

Design.  Each movable joint gets one frame (R, t) in registers.  Links attached by fixed joints
share their moving ancestor's frame; their spheres are re-expressed in that frame at generation
time (float64, then rounded once to float32).  A frame is the parent frame times a constant
transform times the joint motion, with exact zeros and ones folded out, so an axis-aligned joint
costs 12 multiply-adds.  Every floating-point operation is emitted explicitly (fused multiply-add,
multiply, add) so that the CUDA and C versions round identically: the GPU kernels and the CPU
oracle compute bit-identical sphere centres.

The reference's generated kernels compute the same kinematics with a different operation order
(src/impl/vamp/robots/panda.hh:5229-5627), so centres agree with the reference to a few ulp, not
bit for bit; the FP64 FK bounds that difference.
"""
from __future__ import annotations

import argparse
import json
import re
import math
import os
from pathlib import Path

import numpy as np

from .urdf import axis_rotation, rpy_matrix

ROOT = Path(__file__).resolve().parents[2]
MODELS = ROOT / "vamp_gb300" / "robots"
CUDA_OUT = ROOT / "vamp_gb300" / "csrc" / "robots"
C_OUT = ROOT / "oracle" / "port" / "robots"


def f32(v: float) -> float:
    return float(np.float32(v))


def lit32(v: float) -> str:
    v = f32(v)
    if v == 0.0:
        return "0.0f"
    r = repr(v)
    if "e" not in r and "." not in r:
        r += ".0"
    return r + "f"


def lit64(v: float) -> str:
    r = repr(float(v))
    if "e" not in r and "." not in r and "inf" not in r and "nan" not in r:
        r += ".0"
    return r


class Emitter:
    """Emits explicit arithmetic for one target.

    A value is a Python float (a constant, already rounded for the target), a variable name, or a
    variable name prefixed with '-' (its negation, folded into the operation that uses it).
    `snap` folds constants within `snap` of 0 or +-1 to exact values (float targets only).
    """

    def __init__(self, target: str, snap: float):
        self.target = target  # "cuda" | "c32" | "c64"
        self.snap = snap
        self.lines: list[str] = []
        self.n = 0
        self.ty = "double" if target == "c64" else "float"
        self.flops = 0  # floating-point operations emitted (a fused multiply-add counts 2)

    def const(self, v: float) -> float:
        if self.snap:
            if abs(v) < self.snap:
                v = 0.0
            elif abs(v - 1.0) < self.snap:
                v = 1.0
            elif abs(v + 1.0) < self.snap:
                v = -1.0
        return float(v) if self.target == "c64" else f32(v)

    def lit(self, v) -> str:
        return lit64(v) if self.target == "c64" else lit32(v)

    def ref(self, v) -> str:
        if isinstance(v, float):
            return self.lit(v)
        return f"(-{v[1:]})" if v.startswith("-") else v

    def _fma(self, a, b, c) -> str:
        self.flops += 2
        a, b, c = self.ref(a), self.ref(b), self.ref(c)
        if self.target == "cuda":
            return f"__fmaf_rn({a}, {b}, {c})"
        return f"{'fma' if self.target == 'c64' else 'fmaf'}({a}, {b}, {c})"

    def _mul(self, a, b) -> str:
        self.flops += 1
        a, b = self.ref(a), self.ref(b)
        return f"__fmul_rn({a}, {b})" if self.target == "cuda" else f"({a} * {b})"

    def _add(self, a, b) -> str:
        self.flops += 1
        a, b = self.ref(a), self.ref(b)
        return f"__fadd_rn({a}, {b})" if self.target == "cuda" else f"({a} + {b})"

    def assign(self, expr: str, name: str | None = None) -> str:
        if name is None:
            name = f"_v{self.n}"
            self.n += 1
        self.lines.append(f"const {self.ty} {name} = {expr};")
        return name

    @staticmethod
    def _neg(v):
        if isinstance(v, float):
            return -v
        return v[1:] if v.startswith("-") else "-" + v

    def lincomb(self, terms, const=0.0, name=None):
        """Emit const + sum(coef * a * b) for terms (coef, a, b|None).  Returns a value.

        Order: the constant (if non-zero) starts the accumulator, then each product is fused
        in turn; a lone product starts with a multiply.
        """
        prods = []
        c0 = const
        for coef, a, b in terms:
            k = coef
            vs = []
            for x in (a, b):
                if x is None:
                    continue
                if isinstance(x, float):
                    k *= x
                else:
                    if x.startswith("-"):
                        k = -k
                        x = x[1:]
                    vs.append(x)
            k = self.const(k)
            if k == 0.0:
                continue
            if not vs:
                c0 += k
                continue
            prods.append((k, vs))
        c0 = self.const(c0)
        if not prods:
            return c0
        # start the accumulator from a bare variable when there is one (saves an operation)
        if c0 == 0.0:
            for i, (k, vs) in enumerate(prods):
                if len(vs) == 1 and k in (1.0, -1.0):
                    prods.insert(0, prods.pop(i))
                    break

        def operand(k, vs):
            # returns (x, y) with x * y == k * prod(vs); may emit one multiply for 3-factor terms
            if len(vs) == 1:
                if k == 1.0:
                    return None, vs[0]
                if k == -1.0:
                    return None, "-" + vs[0]
                return k, vs[0]
            if k == 1.0:
                return vs[0], vs[1]
            if k == -1.0:
                return "-" + vs[0], vs[1]
            t = self.assign(self._mul(k, vs[0]))
            return t, vs[1]

        if c0 != 0.0:
            acc = c0
            rest = prods
        else:
            x, y = operand(*prods[0])
            if x is None:
                acc = y
            else:
                acc = self.assign(self._mul(x, y))
            rest = prods[1:]
        for k, vs in rest:
            x, y = operand(k, vs)
            if x is None:
                if y.startswith("-"):
                    acc = self.assign(self._add(acc, y))  # acc + (-y)
                else:
                    acc = self.assign(self._add(acc, y))
            else:
                acc = self.assign(self._fma(x, y, acc))
        if name is not None and isinstance(acc, str):
            last = self.lines[-1] if self.lines else ""
            if acc.startswith("_v") and last.startswith(f"const {self.ty} {acc} ="):
                self.lines[-1] = last.replace(f"const {self.ty} {acc} =", f"const {self.ty} {name} =", 1)
                return name
            return self.assign(self.ref(acc), name)
        return acc


# --------------------------------------------------------------------------------------------
# kinematic structure


class Kin:
    """Frames of a robot: one per movable joint plus the root, with fixed links folded."""

    def __init__(self, model: dict):
        self.m = model
        joints = model["joints"]
        self.by_child = {j["child"]: j for j in joints}
        self.jindex = {n: i for i, n in enumerate(model["joint_names"])}
        # frame of every link: (frame_id, constant 4x4 from frame to link)
        self.link_frame = {model["root"]: ("root", np.eye(4))}
        self.frames = []  # movable frames in topological order: dict
        pending = list(joints)
        while pending:
            rest = []
            for j in pending:
                if j["parent"] not in self.link_frame:
                    rest.append(j)
                    continue
                fid, C = self.link_frame[j["parent"]]
                O = np.eye(4)
                O[:3, :3] = rpy_matrix(j["rpy"])
                O[:3, 3] = j["xyz"]
                K = C @ O
                if j["type"] == "fixed" or j["name"] not in self.jindex:
                    if j["type"] != "fixed":
                        # a movable joint the configuration does not drive: hold it at zero
                        pass
                    self.link_frame[j["child"]] = (fid, K)
                else:
                    name = f"F{len(self.frames)}"
                    self.frames.append(
                        {
                            "id": name,
                            "parent": fid,
                            "K": K,
                            "axis": np.asarray(j["axis"], dtype=np.float64),
                            "type": j["type"],
                            "q": self.jindex[j["name"]],
                            "joint": j["name"],
                        }
                    )
                    self.link_frame[j["child"]] = (name, np.eye(4))
            assert len(rest) < len(pending)
            pending = rest

    def sphere_in_frame(self, link: str, p) -> tuple:
        fid, C = self.link_frame[link]
        v = C @ np.array([p[0], p[1], p[2], 1.0])
        return fid, v[:3]


def emit_frames(kin: Kin, em: Emitter, qname="q", sc_fn=None):
    """Emit every movable frame; returns {frame_id: (R, t)} with values (floats or names)."""
    frames = {"root": ([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]], [0.0, 0.0, 0.0])}
    for f in kin.frames:
        Rp, tp = frames[f["parent"]]
        K = f["K"]
        fid = f["id"]
        # fixed part: M = Rp @ K_R, t0 = tp + Rp @ K_t
        t0 = [em.lincomb([(float(K[k, 3]), Rp[r][k], None) for k in range(3)] + [(1.0, tp[r], None)]) for r in range(3)]
        M = [[em.lincomb([(float(K[k, c]), Rp[r][k], None) for k in range(3)]) for c in range(3)] for r in range(3)]
        axis = f["axis"] / np.linalg.norm(f["axis"])
        qv = f"{qname}[{f['q']}]"
        if f["type"] in ("revolute", "continuous"):
            s, c = f"{fid}_s", f"{fid}_c"
            em.lines.append(sc_fn(qv, s, c))
            # joint rotation (Rodrigues): Rj = c (I - a a^T) + s [a]x + a a^T
            kx = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
            aa = np.outer(axis, axis)
            R = []
            for r in range(3):
                row = []
                for cc in range(3):
                    terms = []
                    for k in range(3):
                        terms.append(((1.0 if k == cc else 0.0) - aa[k, cc], M[r][k], c))
                        terms.append((kx[k, cc], M[r][k], s))
                        terms.append((aa[k, cc], M[r][k], None))
                    row.append(em.lincomb(terms, 0.0, name=f"{fid}_r{r}{cc}"))
                R.append(row)
            t = [em.lincomb([(1.0, t0[r], None)], 0.0, name=f"{fid}_t{r}") for r in range(3)]
        elif f["type"] == "prismatic":
            R = M
            t = [
                em.lincomb(
                    [(1.0, t0[r], None)] + [(float(axis[k]), M[r][k], qv) for k in range(3)],
                    0.0,
                    name=f"{fid}_t{r}",
                )
                for r in range(3)
            ]
        else:
            raise ValueError(f["type"])
        frames[fid] = (R, t)
    return frames


def emit_centre(em: Emitter, frames, kin: Kin, link: str, p, prefix: str):
    """Centre of a sphere at offset p of `link`: t + R p, evaluated as t, then one fused
    multiply-add per column of R, for every coordinate.  The frame's entries are used as they
    are (constants are not folded into the chain), so a centre computed from frame values held in
    registers, in local memory or on the CPU rounds identically."""
    fid, v = kin.sphere_in_frame(link, p)
    R, t = frames[fid]
    out = []
    for r in range(3):
        acc = t[r]
        for k in range(3):
            acc = em.assign(em._fma(R[r][k], em.const(float(v[k])), acc))
        last = em.lines[-1]
        name = f"{prefix}{'xyz'[r]}"
        em.lines[-1] = last.replace(f"const {em.ty} {acc} =", f"const {em.ty} {name} =", 1)
        out.append(name)
    return out


def emit_ee_pose(em: Emitter, frames, kin: Kin, link: str):
    """Transform of `link` (the end effector, where fkcc_attach poses the attachment): its
    frame's R and t composed with the constant link offset, R row-major then t, each entry one
    lincomb (the same operation sequence as the frames themselves).  Returns 12 values."""
    fid, C = kin.link_frame[link]
    Rp, tp = frames[fid]
    R = [[em.lincomb([(float(C[k, c]), Rp[r][k], None) for k in range(3)]) for c in range(3)] for r in range(3)]
    t = [em.lincomb([(float(C[k, 3]), Rp[r][k], None) for k in range(3)] + [(1.0, tp[r], None)]) for r in range(3)]
    return [R[r][c] for r in range(3) for c in range(3)] + t


def attach_tables(model: dict, coarse_slot: dict):
    """Per robot link checked against an attachment (fkcc_attach, in the reference's order): its
    coarse slot and the range of its fine slots in the flat fine list."""
    rows, fine = [], []
    for c in model.get("attach_checks", []):
        rows.append((coarse_slot[c["link"]], len(fine), len(fine) + len(c["fine"])))
        fine += c["fine"]
    return rows, fine


# sin_ref + cos_ref of one joint angle: 24 + 25 floating-point operations (vg_check.cuh)
SINCOS_FLOPS = 49
# one sphere centre from its frame: 9 fused multiply-adds
CENTRE_FLOPS = 18


def fk_flops(model: dict) -> dict:
    """Floating-point operations of the generated FP32 kinematics for one configuration."""
    kin = Kin(model)
    em = Emitter("cuda", SNAP32)
    emit_frames(kin, em, "q", sc_fn=lambda x, s_, c: "")
    n_rev = sum(1 for f in kin.frames if f["type"] in ("revolute", "continuous"))
    slots, _ = slot_table(model)
    return {"frames": em.flops + SINCOS_FLOPS * n_rev, "centre": CENTRE_FLOPS, "slots": len(slots)}


def frame_values(kin: Kin, frames) -> list:
    """Every frame (root first, then movable frames in order) as 12 values: R row-major, t."""
    out = []
    for fid in ["root"] + [f["id"] for f in kin.frames]:
        R, t = frames[fid]
        out.append([R[r][c] for r in range(3) for c in range(3)] + list(t))
    return out


def frame_index(kin: Kin) -> dict:
    return {fid: i for i, fid in enumerate(["root"] + [f["id"] for f in kin.frames])}


def struct_name(name: str) -> str:
    return name[0].upper() + name[1:]


def slot_table(model: dict):
    """Slot order: fine spheres 0..n-1 (reference order), then one coarse sphere per env link."""
    slots = [(f["link"], f["p"], f["r"]) for f in model["fine_spheres"]]
    coarse_slot = {}
    for e in model["env_checks"]:
        link = e["link"]
        c = model["coarse_spheres"][link]
        coarse_slot[link] = len(slots)
        slots.append((link, c["p"], c["r"]))
    return slots, coarse_slot


# --------------------------------------------------------------------------------------------
# CUDA output


# Robots whose check schedule is emitted as table-driven loops (frames in local memory) rather
# than straight-line code: their schedules are large enough (hundreds of link pairs) that
# straight-line code spends minutes in ptxas and spills heavily.  Results are identical either way.
TABLED = {"ur5", "fetch", "baxter"}
# FP32 constants this close to 0 or +-1 are folded to exact values: URDF angles such as
# 1.570796325 leave ~1e-9 residues that only cost operations (their effect is below 1e-8 m)
SNAP32 = 1e-7
# Coarse spheres queried together (one pass over the objects, up to the largest bound among
# them): four in the unrolled environment section (one inlined copy per batch), two in the looped
# one (one copy in all), the fastest of 1-11 measured on the Panda's 65,536-edge workload.
COARSE_BATCH = int(os.environ.get("VG_COARSE_BATCH", "4"))
LOOPED_BATCH = int(os.environ.get("VG_LOOPED_BATCH", "2"))


def f32_down(v: float) -> float:
    """Largest float32 <= v (a conservative lower bound in FP32)."""
    x = np.float32(v)
    return float(x) if float(x) <= v else float(np.nextafter(x, np.float32(-np.inf)))


def f32_up(v: float) -> float:
    """Smallest float32 >= v."""
    x = np.float32(v)
    return float(x) if float(x) >= v else float(np.nextafter(x, np.float32(np.inf)))


BIG = 3.0e38  # an unbounded box side (joint values are finite)


def danger_boxes(model: dict, cull) -> tuple:
    """Per self check ((joint indices, index of its first pair box or -1), union box) and the
    boxes of the analysed checks' live pairs, as FP32 bounds rounded outwards; unanalysed checks
    get an unbounded union box and no pair boxes."""
    checks, pairs = [], []
    for ci, e in enumerate(model["self_checks"]):
        bx = None if cull is None or "boxes" not in cull else cull["boxes"][ci]
        sel = range(len(e["fine"])) if cull is None or cull["live"][ci] is None else cull["live"][ci]
        n_live = len(list(sel))
        if not bx:
            checks.append(((0, 0, -1), (-BIG, BIG, -BIG, BIG)))
            continue
        j = bx[0]["joints"]
        two = len(j) == 2
        jj = (j[0], j[1] if two else j[0])
        per = []
        for b in bx:
            lo1, hi1 = (b["lo"][1], b["hi"][1]) if two else (-BIG, BIG)
            per.append((f32_down(b["lo"][0]), f32_up(b["hi"][0]), f32_down(lo1) if two else -BIG, f32_up(hi1) if two else BIG))
        union = (min(p[0] for p in per), max(p[1] for p in per), min(p[2] for p in per), max(p[3] for p in per))
        checks.append(((jj[0], jj[1], len(pairs)), union))
        pairs += per
    return checks, pairs


CONTAIN_MARGIN = 1e-4  # metres between a link's fine spheres and its containing sphere


def containing_radius(model: dict, kin, env_check: dict) -> float:
    """Largest |fine centre - coarse centre| + fine radius of a link, in float64."""
    slots, cslot = slot_table(model)
    link = env_check["link"]
    fc, pc = kin.sphere_in_frame(slots[cslot[link]][0], slots[cslot[link]][1])
    best = 0.0
    for f in env_check["fine"]:
        ff, pf = kin.sphere_in_frame(slots[f][0], slots[f][1])
        assert ff == fc, "a link's fine spheres and its coarse sphere share one frame"
        best = max(best, float(np.linalg.norm(np.asarray(pf, float) - np.asarray(pc, float))) + float(slots[f][2]))
    return best


def load_cull(name: str):
    """Live fine self pairs per self check (None: all live), from robots/<name>.cull.json."""
    path = MODELS / f"{name}.cull.json"
    if not path.exists():
        return None
    return json.loads(path.read_text())


def limits_code(model: dict, cull) -> list:
    """Lines setting ctx.in_limits: every active lane's configuration lies in the joint limits
    widened by the culling slack (the precondition for skipping culled self pairs)."""
    if cull is None:
        return ["ctx.in_limits = false;"]
    slack = cull["slack_rad"]
    lines = ["bool inl = true;"]
    for d, (m_, a_) in enumerate(zip(model["s_m"], model["s_a"])):
        lo = f32(a_ - slack)
        hi = f32(a_ + m_ + slack)
        lines.append(f"inl &= (q[{d}] >= {lit32(lo)}) & (q[{d}] <= {lit32(hi)});")
    lines.append("ctx.in_limits = __all_sync(vg::kFull, inl || !((ctx.alive >> (threadIdx.x & 31)) & 1u));")
    return lines


def _aliases(lines) -> dict:
    """name -> (name, sign) for the emitted copies `const float A = B;` and `const float A = (-B);`."""
    out = {}
    for line in lines:
        m = re.fullmatch(r"const float (\w+) = (?:\(-(\w+)\)|(\w+));", line.strip())
        if m:
            out[m.group(1)] = (m.group(2), -1) if m.group(2) else (m.group(3), 1)
    return out


def stage_layout(model: dict, kin, cull) -> dict:
    """The staged form's shared-memory stage, per thread: each distinct non-constant value among
    the entries of the frames the fine checks use (an entry that is a copy of another takes that
    value's slot), then the centres of every coarse sphere, then the joint values the danger
    boxes test."""
    slots, _ = slot_table(model)
    em = Emitter("cuda", SNAP32)
    fr = emit_frames(kin, em, "q", sc_fn=lambda x, s_, c: "")
    # VG_STAGE_NO_DEDUP=1 (generator switch): one slot per frame entry, copies included
    alias = {} if os.environ.get("VG_STAGE_NO_DEDUP") == "1" else _aliases(em.lines)

    def resolve(name):
        sign = 1
        while name in alias:
            name, sg = alias[name]
            sign *= sg
        return name, sign

    order = []
    for e in model["env_checks"]:
        order.append(kin.sphere_in_frame(slots[e["fine"][0]][0], slots[e["fine"][0]][1])[0])
    for e in model["self_checks"]:
        A, B = _pairs_ab(e)
        order.append(kin.sphere_in_frame(slots[A[0]][0], slots[A[0]][1])[0])
        order.append(kin.sphere_in_frame(slots[B[0]][0], slots[B[0]][1])[0])
    frames, fslots, fconsts, values = {}, [], [], {}
    for fid in order:
        if fid in frames:
            continue
        frames[fid] = len(fslots)
        R, t = fr[fid]
        row_s, row_c = [], []
        for v in [R[r][c] for r in range(3) for c in range(3)] + list(t):
            if isinstance(v, float):
                row_s.append(-1)
                row_c.append(v)
                continue
            neg = v.startswith("-")
            base, sign = resolve(v[1:] if neg else v)
            sign = -sign if neg else sign
            # a negated copy gets its own slot: decoding a sign per entry costs more in the fine
            # checks than the slot saves
            key = base if sign > 0 else "-" + base
            if key not in values:
                values[key] = len(values)
            row_s.append(values[key])
            row_c.append(0.0)
        fslots.append(row_s)
        fconsts.append(row_c)
    n = len(values)
    n_env = len(model["env_checks"])
    checks, _ = danger_boxes(model, cull)
    joints = sorted({j for (j0, j1, b0), _ in checks if b0 >= 0 for j in (j0, j1)}) or [0]
    return {"frames": frames, "slots": fslots, "consts": fconsts, "n_frame": n, "values": list(values),
            "coarse": list(range(n_env)), "coarse_pos": {k: k for k in range(n_env)},
            "joints": joints, "joint_pos": {j: i for i, j in enumerate(joints)},
            "coarse0": n, "q0": n + 3 * n_env, "total": n + 3 * n_env + len(joints)}


def _pairs_ab(e):
    A, B = [], []
    for sa, sb in e["fine"]:
        if sa not in A:
            A.append(sa)
        if sb not in B:
            B.append(sb)
    # the reference's fine pairs for a link pair are the cross product of the two links' spheres
    assert [[x, y] for x in A for y in B] == e["fine"], "fine self pairs are not a cross product"
    return A, B


def gen_cuda(model: dict) -> str:
    name = model["name"]
    S = struct_name(name)
    kin = Kin(model)
    slots, coarse_slot = slot_table(model)
    dim = model["dimension"]
    tabled = name in TABLED
    fidx = frame_index(kin)
    lines = []
    w = lines.append
    w("// Generated by vamp_gb300/robotgen/codegen.py from vamp_gb300/robots/%s.json. Do not edit." % name)
    w("//")
    w("// FP32 forward kinematics and the fkcc check schedule of the %s robot, one configuration" % name)
    w("// per thread.  Schedule order follows the reference's generated Robot::fkcc")
    w("// (src/impl/vamp/robots/%s.hh): environment checks link by link, each a coarse link sphere" % name)
    w("// gating that link's fine spheres, then self-collision link pairs, a coarse pair gating the")
    w("// cross product of the two links' fine spheres.  Schedule form: %s." % ("table-driven loops" if tabled else "straight-line"))
    w("#pragma once")
    w("")
    w('#include "../vg_check.cuh"')
    w("")
    w("namespace vg::robots")
    w("{")

    def frames_block(em):
        return emit_frames(kin, em, "q", sc_fn=lambda x, s_, c: f"float {s_}, {c}; vg_sincos_ref({x}, &{s_}, &{c});")

    # ---- tables (constant memory) for the table-driven form, and slot data for both
    env_start, env_fine = [0], []
    for e in model["env_checks"]:
        env_fine += e["fine"]
        env_start.append(len(env_fine))
    self_rows, self_list = [], []
    for e in model["self_checks"]:
        A, B = _pairs_ab(e)
        a0 = len(self_list)
        self_list += A
        b0 = len(self_list)
        self_list += B
        self_rows.append((coarse_slot[e["links"][0]], coarse_slot[e["links"][1]], a0, b0, len(A), len(B)))
    if True:
        pre = f"k{S}"
        w(f"    // slot -> frame, and the slot's centre offset in that frame and radius")
        w(f"    __constant__ int {pre}SlotFrame[{len(slots)}] = {{{', '.join(str(fidx[kin.sphere_in_frame(l, p)[0]]) for l, p, r in slots)}}};")
        offs = []
        em0 = Emitter("cuda", SNAP32)
        for l, p, r in slots:
            v = kin.sphere_in_frame(l, p)[1]
            offs.append(f"{{{lit32(em0.const(float(v[0])))}, {lit32(em0.const(float(v[1])))}, {lit32(em0.const(float(v[2])))}, {lit32(r)}}}")
        w(f"    __constant__ float4 {pre}SlotOff[{len(slots)}] = {{{', '.join(offs)}}};")
        # tables of the table-driven form: only for the robots that compile that form (and
        # only while VG_STAGED_ALL does not switch them to the staged form)
        w(f"    __constant__ int {pre}EnvStart[{len(env_start)}] = {{{', '.join(map(str, env_start))}}};")
        if tabled:
            w("#ifndef VG_STAGED_ALL")
            w(f"    __constant__ int {pre}EnvCoarse[{len(model['env_checks'])}] = {{{', '.join(str(coarse_slot[e['link']]) for e in model['env_checks'])}}};")
            w("#endif")
        w(f"    __constant__ int {pre}EnvFine[{len(env_fine)}] = {{{', '.join(map(str, env_fine))}}};")
        if tabled:
            w("#ifndef VG_STAGED_ALL")
            w(f"    // per link pair: coarse slot A, coarse slot B, start of A's and B's fine lists, their sizes")
            w(f"    __constant__ int4 {pre}SelfRow[{len(self_rows)}] = {{{', '.join('{%d, %d, %d, %d}' % r[:4] for r in self_rows)}}};")
            w(f"    __constant__ int2 {pre}SelfLen[{len(self_rows)}] = {{{', '.join('{%d, %d}' % r[4:] for r in self_rows)}}};")
            w(f"    __constant__ int {pre}SelfList[{len(self_list)}] = {{{', '.join(map(str, self_list))}}};")
            env_of = {e["link"]: k for k, e in enumerate(model["env_checks"])}
            w(f"    // per link pair: environment-check index of link A's and link B's coarse sphere")
            w(f"    __constant__ int2 {pre}SelfEnvIdx[{len(self_rows)}] = {{{', '.join('{%d, %d}' % (env_of[e['links'][0]], env_of[e['links'][1]]) for e in model['self_checks'])}}};")
            w("#endif")
        cull = load_cull(name)
        live_start, live_pairs = [0], []
        for ci, e in enumerate(model["self_checks"]):
            sel = range(len(e["fine"])) if cull is None or cull["live"][ci] is None else cull["live"][ci]
            live_pairs += [tuple(e["fine"][pi]) for pi in sel]
            live_start.append(len(live_pairs))
        w(f"    // fine pairs that can collide inside the widened joint limits, per self check")
        w(f"    __constant__ int {pre}LiveStart[{len(live_start)}] = {{{', '.join(map(str, live_start))}}};")
        w(f"    __constant__ int2 {pre}LivePair[{max(1, len(live_pairs))}] = {{{', '.join('{%d, %d}' % p for p in live_pairs) or '{0, 0}'}}};")
        all_pairs = [tuple(p_) for e in model["self_checks"] for p_ in e["fine"]]
        w(f"    // every fine self pair, in the reference's order (debug reports; global memory)")
        w(f"    __device__ const int2 {pre}AllPair[{max(1, len(all_pairs))}] = {{{', '.join('{%d, %d}' % p for p in all_pairs) or '{0, 0}'}}};")
        arows, afine = attach_tables(model, coarse_slot)
        w(f"    // links checked against an attachment (fkcc_attach): coarse slot, fine range; fine slots")
        w(f"    __device__ const int4 {pre}AttachLink[{max(1, len(arows))}] = {{{', '.join('{%d, %d, %d, 0}' % r for r in arows) or '{0, 0, 0, 0}'}}};")
        w(f"    __device__ const int {pre}AttachFine[{max(1, len(afine))}] = {{{', '.join(map(str, afine)) or '0'}}};")
        # tables of the staged form: every robot's default except the table-driven ones
        if tabled:
            w("#ifdef VG_STAGED_ALL")
        w(f"    __constant__ int2 {pre}FullPair[{max(1, len(all_pairs))}] = {{{', '.join('{%d, %d}' % p for p in all_pairs) or '{0, 0}'}}};")
        if True:
            lay = stage_layout(model, kin, load_cull(name))
            nfr = len(lay["slots"])
            env_frames = [lay["frames"][kin.sphere_in_frame(slots[e["fine"][0]][0], slots[e["fine"][0]][1])[0]]
                          for e in model["env_checks"]]
            w(f"    // staged frame of each environment check's fine spheres")
            w(f"    __constant__ int {pre}EnvFrameS[{len(env_frames)}] = {{{', '.join(map(str, env_frames))}}};")
            w(f"    // per staged frame and entry: its stage slot, or -1 and the constant value")
            w(f"    __constant__ int {pre}FrameSlot[{nfr}][12] = {{{', '.join('{' + ', '.join(map(str, r)) + '}' for r in lay['slots'])}}};")
            w(f"    __constant__ float {pre}FrameConst[{nfr}][12] = {{{', '.join('{' + ', '.join(lit32(v) for v in r) + '}' for r in lay['consts'])}}};")
            env_ix = {e["link"]: k for k, e in enumerate(model["env_checks"])}
            rows_a, rows_b = [], []
            lvs, fls = 0, 0
            cull1 = load_cull(name)
            for ci, e in enumerate(model["self_checks"]):
                A, B = _pairs_ab(e)
                fa = kin.sphere_in_frame(slots[A[0]][0], slots[A[0]][1])[0]
                fb = kin.sphere_in_frame(slots[B[0]][0], slots[B[0]][1])[0]
                sel = range(len(e["fine"])) if cull1 is None or cull1["live"][ci] is None else cull1["live"][ci]
                nl, nf = len(list(sel)), len(e["fine"])
                rows_a.append((lay["coarse_pos"][env_ix[e["links"][0]]], lay["coarse_pos"][env_ix[e["links"][1]]],
                               lay["frames"][fa], lay["frames"][fb]))
                rows_b.append((lvs, lvs + nl, fls, fls + nf))
                lvs += nl
                fls += nf
            w(f"    // self-check loop: staged coarse centre of link A and B, their staged frames;")
            w(f"    // live pair range, full pair range")
            w(f"    __constant__ int4 {pre}SelfA[{len(rows_a)}] = {{{', '.join('{%d, %d, %d, %d}' % r for r in rows_a)}}};")
            w(f"    __constant__ int4 {pre}SelfB[{len(rows_b)}] = {{{', '.join('{%d, %d, %d, %d}' % r for r in rows_b)}}};")
            w(f"    __constant__ float {pre}CoarseR[{len(lay['coarse'])}] = {{{', '.join(lit32(model['coarse_spheres'][model['env_checks'][k]['link']]['r']) for k in lay['coarse'])}}};")
            w(f"    // per environment-check link: radius about its coarse centre that contains every fine sphere")
            w(f"    // of the link with {CONTAIN_MARGIN} m to spare (exact geometry, rounded up to FP32)")
            w(f"    __constant__ float {pre}ContainR[{len(model['env_checks'])}] = {{{', '.join(lit32(f32_up(containing_radius(model, kin, e) + CONTAIN_MARGIN)) for e in model['env_checks'])}}};")
            cb_checks, cb_pairs = danger_boxes(model, cull1)
            box = lambda b: "{%s}" % ", ".join(lit32(v) for v in b)  # noqa: E731
            w(f"    // danger boxes (joint space, inside the widened limits): a live pair can come within the")
            w(f"    // culling margin only for joint values inside its box; per self check the two joints and")
            w(f"    // the union of its pairs' boxes (and where its live pairs' boxes start, -1: none), per")
            w(f"    // live pair of an analysed check its box (lo0, hi0, lo1, hi1)")
            jp = lay["joint_pos"]
            w(f"    __constant__ int4 {pre}SelfJoint[{len(cb_checks)}] = {{{', '.join('{%d, %d, %d, 0}' % ((jp[c[0][0]], jp[c[0][1]], c[0][2]) if c[0][2] >= 0 else (0, 0, -1)) for c in cb_checks)}}};")
            w(f"    __constant__ float4 {pre}SelfBox[{len(cb_checks)}] = {{{', '.join(box(c[1]) for c in cb_checks)}}};")
            w(f"    __constant__ float4 {pre}LiveBox[{max(1, len(cb_pairs))}] = {{{', '.join(box(p_) for p_ in cb_pairs) or box((0, 0, 0, 0))}}};")
        if tabled:
            w("#endif")
        w("")

    w("struct %s" % S)
    w("{")
    w("    static constexpr const char *kName = \"%s\";" % name)
    w("    static constexpr int kDim = %d;" % dim)
    w("    static constexpr int kFine = %d;" % len(model["fine_spheres"]))
    w("    static constexpr int kSlots = %d;" % len(slots))
    w("    static constexpr int kFrames = %d;" % (len(kin.frames) + 1))
    w("    static constexpr int kEnvChecks = %d;" % len(model["env_checks"]))
    w("    static constexpr int kSelfPairs = %d;" % sum(len(e["fine"]) for e in model["self_checks"]))
    w("    static __device__ __forceinline__ int2 self_pair(int i) { return k%sAllPair[i]; }" % S)
    lay = stage_layout(model, kin, load_cull(name))
    w("    // floats of shared-memory staging per thread (non-constant entries of the fine checks' frames)")
    w("#if defined(VG_FORM_COMPACT)%s" % (" || !defined(VG_STAGED_ALL)" if tabled else ""))
    w("    static constexpr int kStage = 0;")
    w("#elif defined(VG_SELF_UNROLLED)")
    w("    static constexpr int kStage = %d;" % lay["n_frame"])
    w("#else")
    w("    // the coarse centres the self-check loop reads and the joint values its danger boxes test")
    w("    static constexpr int kStage = %d;" % lay["total"])
    w("#endif")
    w("    static constexpr int kResolution = %d;" % model["resolution"])
    w("    static constexpr float kMinRadius = %s;" % lit32(model["min_radius"]))
    w("    static constexpr float kMaxRadius = %s;" % lit32(model["max_radius"]))
    w("    static constexpr float kScaleM[%d] = {%s};" % (dim, ", ".join(lit32(v) for v in model["s_m"])))
    w("    static constexpr float kScaleA[%d] = {%s};" % (dim, ", ".join(lit32(v) for v in model["s_a"])))
    w("")

    # ---- all sphere slots, straight-line (FK queries)
    em = Emitter("cuda", SNAP32)
    fr = frames_block(em)
    body = list(em.lines)
    for i, (link, p, r) in enumerate(slots):
        em.lines = []
        x, y, z = emit_centre(em, fr, kin, link, p, f"s{i}_")
        body += em.lines
        body.append(f"out[{4 * i}] = {x}; out[{4 * i + 1}] = {y}; out[{4 * i + 2}] = {z}; out[{4 * i + 3}] = {lit32(r)};")
    w("    // Every sphere slot: fine spheres 0..kFine-1, then the coarse sphere of each checked link.")
    w("    static __device__ __forceinline__ void spheres(const float *q, float *out)")
    w("    {")
    for l in body:
        w("        " + l)
    w("    }")
    w("")

    # ---- end-effector transform and the attachment checks (fkcc_attach)
    em = Emitter("cuda", SNAP32)
    fr = frames_block(em)
    vals = emit_ee_pose(em, fr, kin, model["end_effector"])
    body = list(em.lines) + [" ".join(f"T[{i}] = {em.ref(v)};" for i, v in enumerate(vals))]
    w(f"    // Transform of {model['end_effector']}, where fkcc_attach poses an attachment: R row-major, then t.")
    w("    static __device__ __forceinline__ void ee_pose(const float *q, float *T)")
    w("    {")
    for l in body:
        w("        " + l)
    w("    }")
    rows, afine = attach_tables(model, coarse_slot)
    w("    // links checked against an attachment, in the reference's order: coarse slot, fine range")
    w(f"    static constexpr int kAttachLinks = {len(rows)};")
    w(f"    static __device__ __forceinline__ int4 attach_link(int i) {{ return k{S}AttachLink[i]; }}")
    w(f"    static __device__ __forceinline__ int attach_fine(int i) {{ return k{S}AttachFine[i]; }}")
    w("")

    if tabled:
        w("#ifndef VG_STAGED_ALL")
        em = Emitter("cuda", SNAP32)
        fr = frames_block(em)
        body = list(em.lines)
        for i, vals in enumerate(frame_values(kin, fr)):
            body.append(" ".join(f"F[{12 * i + j}] = {em.ref(v)};" for j, v in enumerate(vals)))
        w("    // Frames (root first): R row-major then t, 12 floats each.")
        w("    static __device__ __forceinline__ void frames(const float *q, float *F)")
        w("    {")
        for l in body:
            w("        " + l)
        w("    }")
        w("")
        pre = f"k{S}"
        w(f"""    static __device__ __forceinline__ float4 centre(const float *F, int slot)
    {{
        const float *f = F + 12 * {pre}SlotFrame[slot];
        const float4 o = {pre}SlotOff[slot];
        float c[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {{
            float acc = f[9 + r];
            acc = __fmaf_rn(f[3 * r + 0], o.x, acc);
            acc = __fmaf_rn(f[3 * r + 1], o.y, acc);
            acc = __fmaf_rn(f[3 * r + 2], o.z, acc);
            c[r] = acc;
        }}
        return make_float4(c[0], c[1], c[2], o.w);
    }}

    // Robot::fkcc for the lanes of ctx.alive.  Clears the lanes of every segment found in collision.
    template <typename Ctx, bool kLoopedEnv = false>
    static __device__ __forceinline__ void fkcc(const float *q, Ctx &ctx)
    {{
        float F[kFrames * 12];
        frames(q, F);
{chr(10).join("        " + l for l in limits_code(model, load_cull(name)))}
        // coarse centres, computed once: the self loop reads them for every link pair
        float4 CC[{len(model['env_checks'])}];
#pragma unroll 1
        for (int c = 0; c < {len(model['env_checks'])}; ++c)
        {{
            const float4 k = centre(F, {pre}EnvCoarse[c]);
            CC[c] = k;
            unsigned need = ctx.env_hit(k.x, k.y, k.z, k.w, ctx.alive);
#pragma unroll 1
            for (int i = {pre}EnvStart[c]; need && i < {pre}EnvStart[c + 1]; ++i)
            {{
                const float4 s = centre(F, {pre}EnvFine[i]);
                const unsigned hit = ctx.env_hit(s.x, s.y, s.z, s.w, need);
                need &= ~hit;
                if (hit && !ctx.kill(hit))
                {{
                    return;
                }}
            }}
        }}
#pragma unroll 1
        for (int c = 0; c < {len(self_rows)}; ++c)
        {{
            const int4 row = {pre}SelfRow[c];
            const int2 ce = {pre}SelfEnvIdx[c];
            const float4 a = CC[ce.x], b = CC[ce.y];
            unsigned need = ctx.self_hit(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, ctx.alive);
            if (!need)
            {{
                continue;
            }}
            unsigned acc = 0u;
            if (ctx.in_limits)
            {{
#pragma unroll 1
                for (int k = {pre}LiveStart[c]; k < {pre}LiveStart[c + 1]; ++k)
                {{
                    const int2 pr = {pre}LivePair[k];
                    const float4 sa = centre(F, pr.x), sb = centre(F, pr.y);
                    acc |= vg::self_bits(sa.x, sa.y, sa.z, sb.x, sb.y, sb.z, __fadd_rn(sa.w, sb.w));
                }}
            }}
            else
            {{
                const int2 len = {pre}SelfLen[c];
#pragma unroll 1
                for (int i = 0; i < len.x; ++i)
                {{
                    const float4 sa = centre(F, {pre}SelfList[row.z + i]);
#pragma unroll 1
                    for (int j = 0; j < len.y; ++j)
                    {{
                        const float4 sb = centre(F, {pre}SelfList[row.w + j]);
                        acc |= vg::self_bits(sa.x, sa.y, sa.z, sb.x, sb.y, sb.z, __fadd_rn(sa.w, sb.w));
                    }}
                }}
            }}
            const unsigned hit = ctx.vote(acc, need);
            if (hit && !ctx.kill(hit))
            {{
                return;
            }}
        }}
    }}""")
        w("#else")


    # ---- compact and staged schedules.  Both: frames in registers while the kinematics run,
    # coarse link spheres queried together, per-check code unrolled, per-sphere and per-pair work
    # in rolled loops over constant tables.  Compact passes the frames to those loops in
    # registers; staged (the default) writes the frames the fine checks need to shared memory
    # once, so that the call sites pass frame indices and the frames need no registers across
    # the checks (smaller code for the instruction cache, fewer live registers).
    pre = f"k{S}"
    cull = load_cull(name)
    em = Emitter("cuda", SNAP32)
    fr = frames_block(em)
    head = list(em.lines)
    head += limits_code(model, cull)
    fvals = frame_values(kin, fr)
    sid = lay["frames"]

    def frame_expr(fid):
        return "vg::Frame{{" + ", ".join(em.ref(v) for v in fvals[fidx[fid]]) + "}}"

    n_env = len(model["env_checks"])
    env_index = {e["link"]: k for k, e in enumerate(model["env_checks"])}

    def centre(i, tag):
        em.lines = []
        link, p, r = slots[i]
        x, y, z = emit_centre(em, fr, kin, link, p, f"{tag}{i}_")
        return list(em.lines), (x, y, z, lit32(r))

    # coarse spheres of every environment-checked link: queried together, reused by self checks
    coarse = [f"float4 cs[{n_env}];"]
    for k, e in enumerate(model["env_checks"]):
        ls, (x, y, z, r) = centre(coarse_slot[e["link"]], "c")
        coarse.append("{")
        coarse += ["    " + l for l in ls]
        coarse.append(f"    cs[{k}] = make_float4({x}, {y}, {z}, {r});  // {e['link']}")
        coarse.append("}")
    coarse.append(f"unsigned ch[{n_env}];")
    nb = -(-n_env // COARSE_BATCH)
    base = 0
    for bi in range(nb):
        size = n_env // nb + (1 if bi < n_env % nb else 0)
        coarse.append(f"ctx.template env_many<{size}>(cs + {base}, ctx.alive, ch + {base});")
        base += size

    stage = []
    vals_ = [f"(-{v[1:]})" if v.startswith("-") else v for v in lay["values"]]
    for i in range(0, len(vals_), 6):
        stage.append(" ".join(f"st[{j} * vg::kStageStride] = {vals_[j]};" for j in range(i, min(i + 6, len(vals_)))))

    def env_section(staged):
        out = []
        for k, e in enumerate(model["env_checks"]):
            fid = kin.sphere_in_frame(slots[e["fine"][0]][0], slots[e["fine"][0]][1])[0]
            for sidx in e["fine"]:
                assert kin.sphere_in_frame(slots[sidx][0], slots[sidx][1])[0] == fid
            fa = str(sid[fid]) if staged else frame_expr(fid)
            out.append(f"// environment: {e['link']} ({len(e['fine'])} fine spheres)")
            out.append("{")
            out.append(f"    const unsigned need = ch[{k}] & ctx.alive;")
            out.append(f"    if (need)")
            out.append("    {")
            if staged:
                out.append(f"        const unsigned hit = env_fine<Ctx::kW, Ctx::kExt>(ctx.env, st, {fa}, {env_start[k]}, {env_start[k + 1]}, need);")
            else:
                out.append(f"        const unsigned hit = env_fine<Ctx::kW, Ctx::kExt>(ctx.env, {fa}, {env_start[k]}, {env_start[k + 1]}, need);")
            out.append("        if (hit && !ctx.kill(hit)) return;")
            out.append("    }")
            out.append("}")
        return out

    full_start, full_pairs, lv_start, lv_pairs = [0], [], [0], []
    for ci, e in enumerate(model["self_checks"]):
        full_pairs += [tuple(p_) for p_ in e["fine"]]
        full_start.append(len(full_pairs))
        sel = range(len(e["fine"])) if cull is None or cull["live"][ci] is None else cull["live"][ci]
        lv_pairs += [tuple(e["fine"][pi]) for pi in sel]
        lv_start.append(len(lv_pairs))

    def self_section(staged):
        out = []
        for ci, e in enumerate(model["self_checks"]):
            a, b = e["links"]
            A, B = _pairs_ab(e)
            fa = kin.sphere_in_frame(slots[A[0]][0], slots[A[0]][1])[0]
            fb = kin.sphere_in_frame(slots[B[0]][0], slots[B[0]][1])[0]
            ka, kb = env_index[a], env_index[b]
            nl = lv_start[ci + 1] - lv_start[ci]
            out.append(f"// self: {a} vs. {b} ({nl} of {len(e['fine'])} fine pairs can collide inside the limits)")
            out.append("{")
            out.append(f"    const unsigned need = ctx.self_hit(cs[{ka}].x, cs[{ka}].y, cs[{ka}].z, cs[{ka}].w, cs[{kb}].x, cs[{kb}].y, cs[{kb}].z, cs[{kb}].w, ctx.alive);")
            out.append("    if (need)")
            out.append("    {")
            if staged:
                cbc = f"make_float4(cs[{kb}].x, cs[{kb}].y, cs[{kb}].z, {pre}ContainR[{kb}])"
                out.append(f"        const unsigned acc = ctx.in_limits ? self_pairs(st, {sid[fa]}, {sid[fb]}, {pre}LivePair, {lv_start[ci]}, {lv_start[ci + 1]}, {cbc})")
                out.append(f"                                           : self_pairs(st, {sid[fa]}, {sid[fb]}, {pre}FullPair, {full_start[ci]}, {full_start[ci + 1]}, {cbc});")
            else:
                out.append(f"        const unsigned acc = ctx.in_limits ? self_pairs({frame_expr(fa)}, {frame_expr(fb)}, {pre}LivePair, {lv_start[ci]}, {lv_start[ci + 1]})")
                out.append(f"                                           : self_pairs({frame_expr(fa)}, {frame_expr(fb)}, {pre}FullPair, {full_start[ci]}, {full_start[ci + 1]});")
            out.append("        const unsigned hit = ctx.vote(acc, need);")
            out.append("        if (hit && !ctx.kill(hit)) return;")
            out.append("    }")
            out.append("}")
        return out

    compact_body = head + coarse + env_section(False) + self_section(False)
    c0 = lay["coarse0"]
    coarse_stage = [" ".join(f"st[{c0 + 3 * i + j} * vg::kStageStride] = cs[{k}].{'xyz'[j]};" for j in range(3))
                    for i, k in enumerate(lay["coarse"])]
    qb = lay["q0"]
    q_stage = [" ".join(f"st[{qb + i} * vg::kStageStride] = q[{d}];" for i, d in enumerate(lay["joints"]))]
    self_loop = f"""#pragma unroll 1
for (int c = 0; c < {len(model['self_checks'])}; ++c)
{{
    const int4 t = {pre}SelfA[c];
    const float *ca = st + ({c0} + 3 * t.x) * vg::kStageStride;
    const float *cb = st + ({c0} + 3 * t.y) * vg::kStageStride;
    const unsigned need = ctx.self_hit(ca[0], ca[vg::kStageStride], ca[2 * vg::kStageStride], {pre}CoarseR[t.x],
                                       cb[0], cb[vg::kStageStride], cb[2 * vg::kStageStride], {pre}CoarseR[t.y], ctx.alive);
    if (need)
    {{
        const int4 u = {pre}SelfB[c];
        const float4 cbc = make_float4(cb[0], cb[vg::kStageStride], cb[2 * vg::kStageStride], {pre}ContainR[t.y]);
        unsigned acc = 0u;
        if (ctx.in_limits)
        {{
            // live pairs only, and only while some lane's joints lie in the check's danger box
            const int4 jj = {pre}SelfJoint[c];
            const float4 bx = {pre}SelfBox[c];
            const float qa = st[({qb} + jj.x) * vg::kStageStride], qb = st[({qb} + jj.y) * vg::kStageStride];
            const bool in = (qa >= bx.x) & (qa <= bx.y) & (qb >= bx.z) & (qb <= bx.w);
            if (__any_sync(vg::kFull, in))
            {{
                acc = self_pairs_boxed(st, t.z, t.w, u.x, u.y, jj.z, qa, qb, cbc);
            }}
        }}
        else
        {{
            acc = self_pairs(st, t.z, t.w, {pre}FullPair, u.z, u.w, cbc);
        }}
        const unsigned hit = ctx.vote(acc, need);
        if (hit && !ctx.kill(hit)) return;
    }}
}}""".split("\n")
    staged_body = head + ["float *const st = ctx.stage;"] + stage + coarse + env_section(True) + self_section(True)
    cut = next(i for i, l in enumerate(coarse) if l.startswith("unsigned ch["))
    lb = LOOPED_BATCH
    nb = -(-n_env // lb)
    env_loops = f"""// coarse spheres of every environment-checked link, {lb} at a time (one copy of the batched query)
unsigned *const chs = ctx.wsc;
#pragma unroll 1
for (int b = 0; b < {nb}; ++b)
{{
    float4 sp[{lb}];
#pragma unroll
    for (int s = 0; s < {lb}; ++s)
    {{
        const int k = {lb} * b + s;
        // padding sphere: far away with radius -inf, it is never tested and never hits
        sp[s] = k < {n_env} ? make_float4(st[({c0} + 3 * k) * vg::kStageStride], st[({c0} + 3 * k + 1) * vg::kStageStride],
                                          st[({c0} + 3 * k + 2) * vg::kStageStride], {pre}CoarseR[k])
                            : make_float4(1.0e10f, 0.0f, 0.0f, -__int_as_float(0x7f800000));
    }}
    unsigned h[{lb}];
    ctx.template env_many<{lb}>(sp, ctx.alive, h);
#pragma unroll
    for (int s = 0; s < {lb}; ++s)
    {{
        if ({lb} * b + s < {n_env} && (threadIdx.x & 31) == 0)
        {{
            chs[{lb} * b + s] = h[s];  // warp-uniform
        }}
    }}
}}
__syncwarp();
// fine spheres of the links whose coarse sphere hit
#pragma unroll 1
for (int k = 0; k < {n_env}; ++k)
{{
    const unsigned need = chs[k] & ctx.alive;
    if (need)
    {{
        const unsigned hit = env_fine_inline<Ctx::kW, Ctx::kExt>(ctx.env, st, {pre}EnvFrameS[k], {pre}EnvStart[k], {pre}EnvStart[k + 1], need);
        if (hit && !ctx.kill(hit)) return;
    }}
}}""".split("\n")
    # the environment section either as loops (one copy of the batched query: small code) or
    # unrolled (the coarse centres stay in registers: fewer instructions); chosen per kernel
    looped_body = (head + ["float *const st = ctx.stage;"] + stage + q_stage + coarse[:cut]
                   + ["if constexpr (kLoopedEnv)", "{"] + ["    " + l for l in coarse_stage + env_loops] + ["}", "else", "{"]
                   + ["    " + l for l in coarse[cut:] + coarse_stage + env_section(True)] + ["}"]
                   + ["// self-collision link pairs, in the reference's order"] + self_loop)

    w("#ifdef VG_FORM_COMPACT")
    w(f"""    // Fine environment tests of the spheres EnvFine[k0..k1) of one frame, for the segments in
    // `need`: the segments whose block collides.
    template <int W, bool kExt = false>
    static __device__ __noinline__ unsigned env_fine(const vg::EnvView &ev, const vg::Frame f, int k0, int k1, unsigned need)
    {{
        unsigned dead = 0u;
#pragma unroll 1
        for (int k = k0; k < k1; ++k)
        {{
            const float4 o = {pre}SlotOff[{pre}EnvFine[k]];
            const float4 c = vg::frame_point(f, o);
            const unsigned hit = vg::env_query_inline<W, kExt>(ev, c.x, c.y, c.z, c.w, need);
            dead |= hit;
            need &= ~hit;
            if (!need)
            {{
                break;
            }}
        }}
        return dead;
    }}

    // OR of the sign bits of the fine self-collision tests of pairs[k0..k1) (slot ids), the first
    // slot of each pair in frame a, the second in frame b.
    static __device__ __noinline__ unsigned self_pairs(const vg::Frame a, const vg::Frame b, const int2 *pairs, int k0, int k1)
    {{
        unsigned acc = 0u;
        int last = -1;
        float4 ca = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll 1
        for (int k = k0; k < k1; ++k)
        {{
            const int2 pr = pairs[k];
            if (pr.x != last)
            {{
                ca = vg::frame_point(a, {pre}SlotOff[pr.x]);
                last = pr.x;
            }}
            const float4 cb = vg::frame_point(b, {pre}SlotOff[pr.y]);
            acc |= vg::self_bits(ca.x, ca.y, ca.z, cb.x, cb.y, cb.z, __fadd_rn(ca.w, cb.w));
        }}
        return acc;
    }}
""")
    w("    // Robot::fkcc for the lanes of ctx.alive.  Clears the lanes of every segment found in collision.")
    w("    template <typename Ctx, bool kLoopedEnv = false>")
    w("    static __device__ __forceinline__ void fkcc(const float *q, Ctx &ctx)")
    w("    {")
    for l in compact_body:
        w("        " + l)
    w("    }")
    w("#else")
    w(f"""    // Staged frame f: its non-constant entries from this thread's stage, the rest constants.
    static __device__ __forceinline__ vg::Frame frame_at(const float *st, int f)
    {{
        vg::Frame r;
#pragma unroll
        for (int c = 0; c < 12; ++c)
        {{
            const int slot = {pre}FrameSlot[f][c];
            r.m[c] = slot >= 0 ? st[slot * vg::kStageStride] : {pre}FrameConst[f][c];
        }}
        return r;
    }}

    // Fine environment tests of the spheres EnvFine[k0..k1) of staged frame f, for the segments
    // in `need`: the segments whose block collides.
    template <int W, bool kExt = false>
    static __device__ __noinline__ unsigned env_fine(const vg::EnvView &ev, const float *st, int f, int k0, int k1, unsigned need)
    {{
        return env_fine_inline<W, kExt>(ev, st, f, k0, k1, need);
    }}

    // The same, inlined into its caller (the looped environment section calls it from one place).
    template <int W, bool kExt = false>
    static __device__ __forceinline__ unsigned env_fine_inline(const vg::EnvView &ev, const float *st, int f, int k0, int k1,
                                                               unsigned need)
    {{
        const vg::Frame fr = frame_at(st, f);
        unsigned dead = 0u;
#pragma unroll 1
        for (int k = k0; k < k1; ++k)
        {{
            const float4 o = {pre}SlotOff[{pre}EnvFine[k]];
            const float4 c = vg::frame_point(fr, o);
            const unsigned hit = vg::env_query_inline<W, kExt>(ev, c.x, c.y, c.z, c.w, need);
            dead |= hit;
            need &= ~hit;
            if (!need)
            {{
                break;
            }}
        }}
        return dead;
    }}

    // OR of the sign bits of the fine self-collision tests of pairs[k0..k1) (slot ids), the first
    // slot of each pair in staged frame fa, the second in staged frame fb.
    // A's fine sphere ca against B's containing sphere cbc (every fine sphere of B lies inside it
    // with CONTAIN margin to spare): whether any lane's sphere may touch one of B's fine spheres.
    // Where no lane's does, the pair tests of this sphere have clear sign bits and are skipped.
    static __device__ __forceinline__ bool row_may_hit(const float4 ca, const float4 cbc)
    {{
        const float dx = __fsub_rn(ca.x, cbc.x), dy = __fsub_rn(ca.y, cbc.y), dz = __fsub_rn(ca.z, cbc.z);
        const float rr = __fadd_rn(ca.w, cbc.w);
        return __any_sync(vg::kFull, __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))) < __fmul_rn(rr, rr));
    }}

    static __device__ __noinline__ unsigned self_pairs(const float *st, int fa, int fb, const int2 *pairs, int k0, int k1,
                                                       float4 cbc)
    {{
        const vg::Frame a = frame_at(st, fa), b = frame_at(st, fb);
        unsigned acc = 0u;
        int last = -1;
        bool row = false;
        float4 ca = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll 1
        for (int k = k0; k < k1; ++k)
        {{
            const int2 pr = pairs[k];
            if (pr.x != last)
            {{
                ca = vg::frame_point(a, {pre}SlotOff[pr.x]);
                last = pr.x;
                row = row_may_hit(ca, cbc);
            }}
            if (!row)
            {{
                continue;
            }}
            const float4 cb = vg::frame_point(b, {pre}SlotOff[pr.y]);
            acc |= vg::self_bits(ca.x, ca.y, ca.z, cb.x, cb.y, cb.z, __fadd_rn(ca.w, cb.w));
        }}
        return acc;
    }}

    // The same over the live pairs LivePair[k0..k1), skipping a pair when no lane's joint values
    // (qa, qb: the check's two joints) lie in its danger box LiveBox[box0 + k - k0] (box0 < 0:
    // the check has no boxes): outside it the pair keeps the culling margin, so its test value
    // cannot be negative.  Warp-uniform; all 32 lanes call.
    static __device__ __noinline__ unsigned self_pairs_boxed(const float *st, int fa, int fb, int k0, int k1, int box0,
                                                             float qa, float qb, float4 cbc)
    {{
        const vg::Frame a = frame_at(st, fa), b = frame_at(st, fb);
        unsigned acc = 0u;
        int last = -1;
        bool row = false;
        float4 ca = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll 1
        for (int k = k0; k < k1; ++k)
        {{
            if (box0 >= 0)
            {{
                const float4 bx = {pre}LiveBox[box0 + k - k0];
                if (!__any_sync(vg::kFull, (qa >= bx.x) & (qa <= bx.y) & (qb >= bx.z) & (qb <= bx.w)))
                {{
                    continue;
                }}
            }}
            const int2 pr = {pre}LivePair[k];
            if (pr.x != last)
            {{
                ca = vg::frame_point(a, {pre}SlotOff[pr.x]);
                last = pr.x;
                row = row_may_hit(ca, cbc);
            }}
            if (!row)
            {{
                continue;
            }}
            const float4 cb = vg::frame_point(b, {pre}SlotOff[pr.y]);
            acc |= vg::self_bits(ca.x, ca.y, ca.z, cb.x, cb.y, cb.z, __fadd_rn(ca.w, cb.w));
        }}
        return acc;
    }}
""")
    w("    // Robot::fkcc for the lanes of ctx.alive.  Clears the lanes of every segment found in collision.")
    w("    template <typename Ctx, bool kLoopedEnv = false>")
    w("    static __device__ __forceinline__ void fkcc(const float *q, Ctx &ctx)")
    w("    {")
    w("#ifdef VG_SELF_UNROLLED")
    for l in staged_body:
        w("        " + l)
    w("#else")
    for l in looped_body:
        w("        " + l)
    w("#endif")
    w("    }")
    w("#endif")
    if tabled:
        w("#endif  // VG_STAGED_ALL")
    w("};")
    w("}  // namespace vg::robots")
    return "\n".join(lines) + "\n"


# --------------------------------------------------------------------------------------------
# C oracle output


def gen_c(model: dict) -> str:
    name = model["name"]
    kin = Kin(model)
    slots, coarse_slot = slot_table(model)
    dim = model["dimension"]
    P = name.upper()
    lines = []
    w = lines.append
    w("/* Generated by vamp_gb300/robotgen/codegen.py from vamp_gb300/robots/%s.json. Do not edit." % name)
    w(" *")
    w(" * CPU oracle tables and kinematics for the %s robot.  Test infrastructure only." % name)
    w(" * Schedule: the reference's Robot::fkcc (src/impl/vamp/robots/%s.hh), as tables." % name)
    w(" * FK: the same FP32 operation sequence as the CUDA kernels, plus an FP64 version. */")
    w("#pragma once")
    w("#include <math.h>")
    w('#include "../vgo_math.h"')
    w("")
    w("#define VGO_%s_DIM %d" % (P, dim))
    w("#define VGO_%s_FINE %d" % (P, len(model["fine_spheres"])))
    w("#define VGO_%s_SLOTS %d" % (P, len(slots)))
    w("#define VGO_%s_RESOLUTION %d" % (P, model["resolution"]))
    w("static const float vgo_%s_s_m[%d] = {%s};" % (name, dim, ", ".join(lit32(v) for v in model["s_m"])))
    w("static const float vgo_%s_s_a[%d] = {%s};" % (name, dim, ", ".join(lit32(v) for v in model["s_a"])))
    w("static const float vgo_%s_radius_range[2] = {%s, %s};" % (name, lit32(model["min_radius"]), lit32(model["max_radius"])))
    # env schedule
    env_coarse = [coarse_slot[e["link"]] for e in model["env_checks"]]
    env_start, env_fine = [], []
    for e in model["env_checks"]:
        env_start.append(len(env_fine))
        env_fine += e["fine"]
    env_start.append(len(env_fine))
    w("#define VGO_%s_ENV_CHECKS %d" % (P, len(env_coarse)))
    w("static const int vgo_%s_env_coarse[] = {%s};" % (name, ", ".join(map(str, env_coarse))))
    w("static const int vgo_%s_env_start[] = {%s};" % (name, ", ".join(map(str, env_start))))
    w("static const int vgo_%s_env_fine[] = {%s};" % (name, ", ".join(map(str, env_fine))))
    self_coarse, self_start, self_fine = [], [], []
    for e in model["self_checks"]:
        a, b = e["links"]
        self_coarse += [coarse_slot[a], coarse_slot[b]]
        self_start.append(len(self_fine) // 2)
        for sa, sb in e["fine"]:
            self_fine += [sa, sb]
    self_start.append(len(self_fine) // 2)
    arows, afine = attach_tables(model, coarse_slot)
    w("#define VGO_%s_ATTACH_LINKS %d" % (P, len(arows)))
    w("static const int vgo_%s_attach_coarse[] = {%s};" % (name, ", ".join(str(r[0]) for r in arows) or "0"))
    w("static const int vgo_%s_attach_start[] = {%s};" % (name, ", ".join(str(r[1]) for r in arows + [(0, len(afine), 0)])))
    w("static const int vgo_%s_attach_fine[] = {%s};" % (name, ", ".join(map(str, afine)) or "0"))
    w("#define VGO_%s_SELF_CHECKS %d" % (P, len(model["self_checks"])))
    w("static const int vgo_%s_self_coarse[] = {%s};" % (name, ", ".join(map(str, self_coarse)) or "0"))
    w("static const int vgo_%s_self_start[] = {%s};" % (name, ", ".join(map(str, self_start))))
    w("static const int vgo_%s_self_fine[] = {%s};" % (name, ", ".join(map(str, self_fine)) or "0"))
    w("")

    for tgt, ty, sc in (("c32", "float", "vgo_sincos_ref"), ("c64", "double", None)):
        em = Emitter(tgt, SNAP32 if tgt == "c32" else 0.0)
        if tgt == "c32":
            scf = lambda x, s, c: f"float {s}, {c}; vgo_sincos_ref({x}, &{s}, &{c});"
        else:
            scf = lambda x, s, c: f"const double {s} = sin({x}), {c} = cos({x});"
        fr = emit_frames(kin, em, "q", sc_fn=scf)
        body = list(em.lines)
        for i, (link, p, r) in enumerate(slots):
            em.lines = []
            x, y, z = emit_centre(em, fr, kin, link, p, f"s{i}_")
            body += em.lines
            rr = lit32(r) if tgt == "c32" else lit64(f32(r))
            body.append(f"out[{4 * i}] = {em.ref(x)}; out[{4 * i + 1}] = {em.ref(y)}; out[{4 * i + 2}] = {em.ref(z)}; out[{4 * i + 3}] = {rr};")
        suffix = "f32" if tgt == "c32" else "f64"
        if tgt == "c32":
            em2 = Emitter(tgt, SNAP32)
            fr2 = emit_frames(kin, em2, "q", sc_fn=scf)
            vals = emit_ee_pose(em2, fr2, kin, model["end_effector"])
            w(f"/* Transform of {model['end_effector']} (fkcc_attach's attachment frame): R row-major, then t. */")
            w(f"static void vgo_{name}_ee_pose_f32(const float *q, float *T)")
            w("{")
            for l in em2.lines:
                w("    " + l)
            w("    " + " ".join(f"T[{i}] = {em2.ref(v)};" for i, v in enumerate(vals)))
            w("}")
            w("")
        w(f"/* Every sphere slot (fine, then coarse), {ty}: out[4 * slot + (x, y, z, r)]. */")
        w(f"static void vgo_{name}_spheres_{suffix}(const {ty} *q, {ty} *out)")
        w("{")
        for l in body:
            w("    " + l)
        w("}")
        w("")
    return "\n".join(lines) + "\n"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("robots", nargs="*", default=["panda", "ur5", "fetch", "baxter"])
    a = ap.parse_args()
    CUDA_OUT.mkdir(parents=True, exist_ok=True)
    C_OUT.mkdir(parents=True, exist_ok=True)
    for r in a.robots:
        model = json.loads((MODELS / f"{r}.json").read_text())
        (CUDA_OUT / f"{r}.cuh").write_text(gen_cuda(model))
        (C_OUT / f"{r}.h").write_text(gen_c(model))
        print(r, "ok")


if __name__ == "__main__":
    main()
