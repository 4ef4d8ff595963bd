"""The allocation-free edge check, vg_validate_motions_device_noalloc, through the C ABI.

Some callers cannot allocate GPU memory while they run: a real-time planner that reserves all
memory up front so that a check can never block on the allocator or fail for lack of memory
mid-plan, or a framework that owns device memory through its own pool.  This entry point keeps
its only scratch (the edge kernel's work counter) in a fixed array inside the library.  Two
calls in a row must both give exactly the ordinary entry point's verdicts and block counts: the
second call sees the counter the first one left behind, so this also checks that it is cleared.
This file is collected last so that a failure here comes after every other test has run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# (schedule, extended): the robot's default schedule and every other one; and an environment with
# a heightfield, which runs the extended segment-per-edge kernel
CASES = [(None, False), (0, False), (1, False), (2, False), (3, False), (None, True)]


@pytest.mark.parametrize("schedule,extended", CASES)
def test_noalloc_edge_check_matches_the_ordinary_entry_point_twice(schedule, extended):
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    rb = vg.panda
    scene = scenes.scene_config1(1)
    if extended:
        scene["heightfields"] = [scenes.heightfield(6)]
    env = vg.Environment.from_scene(scene)
    if schedule is not None:
        env.set_schedule(schedule)
    a, b = scenes.edges(rb.s_m, rb.s_a, 16384, 606)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    stream = torch.cuda.current_stream().cuda_stream

    # the ordinary entry point (it also uploads the environment to this GPU)
    ref = torch.empty(len(a), dtype=torch.uint8, device="cuda")
    ref_blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    assert lib.vg_validate_motions_device(b"panda", env.handle, da.data_ptr(), db.data_ptr(), len(a), 32,
                                          ref.data_ptr(), ref_blocks.data_ptr(), stream) == 0

    for call in range(2):
        out = torch.full((len(a),), 7, dtype=torch.uint8, device="cuda")
        blocks = torch.full((len(a),), -1, dtype=torch.int32, device="cuda")
        rc = lib.vg_validate_motions_device_noalloc(b"panda", env.handle, da.data_ptr(), db.data_ptr(), len(a), 32,
                                                    out.data_ptr(), blocks.data_ptr(), stream)
        assert rc == 0, lib.vg_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, ref), f"verdicts differ on call {call + 1}"
        assert torch.equal(blocks, ref_blocks), f"block counts differ on call {call + 1}"
    assert 0 < int(ref.sum()) < len(a)


def test_noalloc_edge_check_refuses_an_environment_not_on_the_gpu():
    import torch

    import vamp_gb300 as vg
    from vamp_gb300._lib import lib

    env = vg.Environment()
    env.add_sphere([1.0, 0.0, 0.5, 0.1])
    q = torch.zeros((4, 7), dtype=torch.float32, device="cuda")
    out = torch.zeros(4, dtype=torch.uint8, device="cuda")
    rc = lib.vg_validate_motions_device_noalloc(b"panda", env.handle, q.data_ptr(), q.data_ptr(), 4, 32, out.data_ptr(),
                                                None, torch.cuda.current_stream().cuda_stream)
    assert rc == -4
    assert b"not uploaded" in lib.vg_last_error()
