"""Failures made on purpose, none of which faults, traps or hangs a GPU.

Host side (no GPU needed): oversized batches and bad handles are refused with an error code
before any GPU work, and configurations outside the joint limits (NaN included) are reported
invalid by the bounds-checked Python calls, as the reference's bindings do
(bindings/robot_helper.hh:256-290).

GPU side: a tensor-core kernel whose MMA-completion wait is given no polls gives up at once; it
waits (with the normal limit) for the MMAs it issued, frees its tensor memory and returns, the
handle reports VG_ERR_CUDA once, and the next call on the same handle runs normally.  An
environment too large for shared memory is refused with VG_ERR_LIMIT.  NaN and infinite
configurations finish (the edge kernels compute at least one block for a NaN length, where the
reference's block count from a NaN length never ends its loop)."""
import ctypes

import numpy as np
import pytest

ERR_ARG, ERR_CUDA, ERR_LIMIT = -1, -2, -5


def test_oversized_batches_are_refused_before_any_gpu_work():
    import vamp_gb300 as vg
    from vamp_gb300._lib import lib

    env = vg.Environment()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    n = 1 << 31
    assert lib.vg_validate_motions_device_noalloc(b"panda", env.handle, dummy, dummy, n, 32, dummy, None, None) == ERR_LIMIT
    assert b"2^31" in lib.vg_last_error()
    assert lib.vg_validate_motions_device(b"panda", env.handle, dummy, dummy, n, 32, dummy, None, None) == ERR_LIMIT
    assert lib.vg_validate_vectors_device(b"panda", env.handle, dummy, dummy, dummy, n, 32, dummy, None, None) == ERR_LIMIT


def test_bad_arguments_are_refused():
    import vamp_gb300 as vg
    from vamp_gb300._lib import lib

    env = vg.Environment()
    assert lib.vg_mlp_set_wait_limit(None, 0) == ERR_ARG
    assert lib.vg_mlp_error(None) == ERR_ARG
    assert lib.vg_fkcc_blocks(b"panda", None, None, 0, None) == ERR_ARG
    assert lib.vg_validate_motions_device(b"panda", env.handle, None, None, 4, 32, None, None, None) == ERR_ARG
    assert lib.vg_validate_motions_device(b"panda", env.handle, None, None, 0, 0, None, None, None) == ERR_ARG  # resolution 0
    assert lib.vg_env_add_heightfield_fields(env.handle, None, 4, 4, None) == ERR_ARG
    big = np.zeros(16, np.float32)
    assert lib.vg_env_add_heightfield_fields(env.handle, big.ctypes.data, 1 << 13, 1 << 12, big.ctypes.data) == ERR_LIMIT


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf, 100.0])
def test_bounds_checked_calls_report_out_of_limit_configurations_invalid(bad):
    import vamp_gb300 as vg

    env = vg.Environment()
    q = (vg.panda.s_a + 0.5 * vg.panda.s_m).astype(np.float32)
    q_bad = q.copy()
    q_bad[2] = bad
    assert vg.panda.validate(q_bad, env, check_bounds=True) is False
    assert vg.panda.validate_motion(q, q_bad, env) is False  # check_bounds defaults to True here


@pytest.mark.gpu
def test_a_tensor_core_wait_that_runs_out_is_reported_once_and_the_handle_recovers():
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    q = torch.from_numpy(scenes.configurations(vg.panda.s_m, vg.panda.s_a, 4096, 21)).cuda()
    m = lib.vg_mlp_create(7, 4)
    try:
        want = torch.empty(4096, dtype=torch.float32, device="cuda")
        assert lib.vg_mlp_infer_device(m, q.data_ptr(), 4096, want.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert lib.vg_mlp_error(m) == 0

        assert lib.vg_mlp_set_wait_limit(m, 0) == 0  # every MMA wait gives up at once
        got = torch.full((4096,), -7.0, dtype=torch.float32, device="cuda")
        assert lib.vg_mlp_infer_device(m, q.data_ptr(), 4096, got.data_ptr(), None) == 0  # the launch itself is fine
        torch.cuda.synchronize()  # the kernel returned: no hang, the context is usable
        assert lib.vg_mlp_error(m) == ERR_CUDA
        assert b"gave up" in lib.vg_last_error()
        assert lib.vg_mlp_error(m) == 0  # reported once

        # the training path (separate GEMM launches) reports it directly
        valid = torch.ones(256, dtype=torch.uint8, device="cuda")
        count = lib.vg_mlp_param_count(7)
        grads = np.zeros(count, np.float32)
        loss = np.zeros(1, np.float32)
        assert lib.vg_mlp_gradients(m, q.data_ptr(), valid.data_ptr(), 256, grads.ctypes.data, loss.ctypes.data, None) == ERR_CUDA
        assert lib.vg_mlp_error(m) == ERR_CUDA and lib.vg_mlp_error(m) == 0

        assert lib.vg_mlp_set_wait_limit(m, -1) == 0  # back to the default
        again = torch.empty(4096, dtype=torch.float32, device="cuda")
        assert lib.vg_mlp_infer_device(m, q.data_ptr(), 4096, again.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert lib.vg_mlp_error(m) == 0
        assert torch.equal(again, want)
        assert lib.vg_mlp_gradients(m, q.data_ptr(), valid.data_ptr(), 256, grads.ctypes.data, loss.ctypes.data, None) == 0
        assert np.all(np.isfinite(grads)) and np.isfinite(loss[0])
    finally:
        lib.vg_mlp_destroy(m)


@pytest.mark.gpu
def test_an_environment_too_large_for_shared_memory_is_refused():
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    rng = np.random.default_rng(3)
    env = vg.Environment()
    for c in rng.uniform(2.0, 3.0, (16000, 3)).astype(np.float32):  # 32 bytes each in shared memory
        env.add_sphere([*c, 0.01])
    q = torch.from_numpy(scenes.configurations(vg.panda.s_m, vg.panda.s_a, 64, 22)).cuda()
    out = torch.empty(64, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.vg_validate_states_device(b"panda", env.handle, q.data_ptr(), 64, out.data_ptr(), s) == ERR_LIMIT
    assert b"shared memory" in lib.vg_last_error()
    assert lib.vg_validate_motions_device(b"panda", env.handle, q.data_ptr(), q.data_ptr(), 64, 32, out.data_ptr(), None,
                                          s) == ERR_LIMIT
    blocks = q[:64].reshape(8, 8, 7).contiguous()
    assert lib.vg_fkcc_blocks_device(b"panda", env.handle, blocks.data_ptr(), 8, out.data_ptr(), s) == ERR_LIMIT
    torch.cuda.synchronize()
    # the library stays usable
    small = vg.Environment.from_scene(scenes.scene_config0(0))
    assert vg.panda.validate_batch(q, small).shape == (64,)


@pytest.mark.gpu
def test_nan_and_infinite_configurations_finish():
    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    env = vg.Environment.from_scene(scenes.scene_config1(1))
    q = scenes.configurations(vg.panda.s_m, vg.panda.s_a, 256, 23)
    q[::3, 4] = np.nan
    q[1::5, 0] = np.inf
    v = vg.panda.validate_batch(q, env)
    assert v.shape == (256,) and set(np.unique(v)) <= {0, 1}
    a, b = q[:128], q[128:]
    e = vg.panda.validate_motion_batch(a, b, env, 32)
    assert e.shape == (128,) and set(np.unique(e)) <= {0, 1}
