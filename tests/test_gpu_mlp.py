"""Tensor-core (tcgen05) kernels of the learned block ordering, against FP32 references."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch

    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (256, 256, 256), (384, 48, 144), (128, 256, 4096)])
def test_bf16_gemm_matches_fp32_reference(torch, M, N, K):
    from vamp_gb300._lib import lib

    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    a = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    d = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.vg_gemm_bf16_device(a.data_ptr(), b.data_ptr(), d.data_ptr(), M, N, K, err.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.vg_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = (a.float().cpu().double() @ b.float().cpu().double().T)
    diff = (d.cpu().double() - ref).abs().max().item()
    scale = ref.abs().max().item()
    assert diff <= 1e-5 * scale * (K ** 0.5), (diff, scale)


# ------------------------------------------------------------------------------- the MLP


def _labelled(torch, n, seed, scene_seed=1):
    """n uniform Panda configurations in the 60-primitive scene with the exact checker's verdicts."""
    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    env = vg.Environment.from_scene(scenes.scene_config1(scene_seed))
    q = scenes.configurations(vg.panda.s_m, vg.panda.s_a, n, seed)
    dq = torch.from_numpy(q).cuda()
    valid = torch.empty(n, dtype=torch.uint8, device="cuda")
    assert lib.vg_validate_states_device(b"panda", env.handle, dq.data_ptr(), n, valid.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    return env, q, dq, valid


def test_mlp_gradients_match_the_cpu_oracle(torch):
    from oracle import mlp
    from vamp_gb300._lib import lib

    dim, n = 7, 1000  # not a multiple of 128: padded rows must contribute nothing
    m = lib.vg_mlp_create(dim, 11)
    assert m
    try:
        _, q, dq, valid = _labelled(torch, n, 77)
        count = lib.vg_mlp_param_count(dim)
        assert count == mlp.param_count(dim)
        params = np.zeros(count, np.float32)
        assert lib.vg_mlp_get_params(m, params.ctypes.data) == 0
        grads = np.zeros(count, np.float32)
        loss = np.zeros(1, np.float32)
        feats = np.zeros((n, mlp.kin_of(dim)), np.float32)
        rc = lib.vg_mlp_gradients(m, dq.data_ptr(), valid.data_ptr(), n, grads.ctypes.data, loss.ctypes.data,
                                  feats.ctypes.data)
        assert rc == 0, lib.vg_last_error()
        # features: BF16 of sin/cos (CUDA sinf/cosf against numpy: within one BF16 step)
        assert np.all(np.abs(feats - mlp.features(q, dim)) <= 2.0 ** -7 * np.abs(mlp.features(q, dim)))
        ref_loss, ref = mlp.loss_and_gradients(params, feats, valid.cpu().numpy(), dim)
        assert abs(loss[0] - ref_loss) <= 1e-5 * max(1.0, abs(ref_loss)), (loss[0], ref_loss)
        # tolerance: FP32 accumulation against float64, plus rare BF16 rounding-boundary flips of
        # intermediate activations; per parameter block, relative to the block's largest gradient
        o = 0
        for name, size in [("W1", 256 * 16), ("b1", 256), ("W2", 256 * 256), ("b2", 256), ("w3", 256), ("b3", 1)]:
            g, r = grads[o:o + size].astype(np.float64), ref[o:o + size]
            o += size
            scale = max(np.abs(r).max(), 1e-12)
            assert np.abs(g - r).max() <= 2e-3 * scale, (name, np.abs(g - r).max(), scale)
            assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r) + 1e-12, name
    finally:
        lib.vg_mlp_destroy(m)


def test_fused_inference_matches_the_training_forward_and_the_oracle(torch):
    from oracle import mlp
    from vamp_gb300 import scenes
    import vamp_gb300 as vg
    from vamp_gb300._lib import lib

    dim, n = 7, 5000
    m = lib.vg_mlp_create(dim, 5)
    try:
        q = scenes.configurations(vg.panda.s_m, vg.panda.s_a, n, 8)
        dq = torch.from_numpy(q).cuda()
        p1 = torch.empty(n, dtype=torch.float32, device="cuda")
        p2 = torch.empty(n, dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        assert lib.vg_mlp_predict_device(m, dq.data_ptr(), n, p1.data_ptr(), s) == 0, lib.vg_last_error()
        assert lib.vg_mlp_infer_device(m, dq.data_ptr(), n, p2.data_ptr(), s) == 0, lib.vg_last_error()
        torch.cuda.synchronize()
        assert lib.vg_mlp_error(m) == 0
        params = np.zeros(mlp.param_count(dim), np.float32)
        lib.vg_mlp_get_params(m, params.ctypes.data)
        ref = mlp.forward(params, mlp.bf16(mlp.features(q, dim)), dim)["p"]
        a, b = p1.cpu().numpy(), p2.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-4, np.abs(a - b).max()
        # the features differ from numpy's sin/cos by BF16 rounding at most, so compare loosely
        assert np.abs(b - ref).max() <= 2e-2, np.abs(b - ref).max()
        assert np.mean(np.abs(b - ref)) <= 2e-3
    finally:
        lib.vg_mlp_destroy(m)


@pytest.fixture(scope="module")
def trained(torch):
    """A Panda MLP trained on 262,144 exact labels of the 60-primitive scene."""
    from vamp_gb300._lib import lib

    env, q, dq, valid = _labelled(torch, 262144, 123)
    m = lib.vg_mlp_create(7, 3)
    losses = np.zeros(4, np.float32)
    rc = lib.vg_mlp_train_device(m, dq.data_ptr(), valid.data_ptr(), len(q), 4, 1024, 1e-3, losses.ctypes.data,
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.vg_last_error()
    yield m, env, losses
    lib.vg_mlp_destroy(m)


def test_training_lowers_the_loss_and_separates_colliding_states(torch, trained):
    from oracle import mlp
    from vamp_gb300._lib import lib

    m, env, losses = trained
    assert np.all(np.isfinite(losses))
    assert losses[-1] < losses[0] < 0.7, losses
    _, q, dq, valid = _labelled(torch, 65536, 999)  # held out
    p = torch.empty(len(q), dtype=torch.float32, device="cuda")
    assert lib.vg_mlp_infer_device(m, dq.data_ptr(), len(q), p.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    auc = mlp.auc(p.cpu().numpy(), valid.cpu().numpy() == 0)
    assert auc > 0.85, auc


def test_learned_order_keeps_every_verdict_and_checks_fewer_blocks(torch, trained):
    from vamp_gb300 import scenes
    import vamp_gb300 as vg
    from vamp_gb300._lib import lib

    m, env, _ = trained
    a, b = scenes.edges(vg.panda.s_m, vg.panda.s_a, 32768, 4242)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    s = torch.cuda.current_stream().cuda_stream
    n = len(a)

    def run(fn, *extra):
        out = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
        blocks = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        rc = fn(b"panda", env.handle, *extra, out.data_ptr(), blocks.data_ptr(), s)
        assert rc == 0, lib.vg_last_error()
        torch.cuda.synchronize()
        return out.cpu().numpy(), blocks.cpu().numpy()

    env.set_schedule(1)
    plain, plain_blocks = run(lambda r, e, o, bl, st: lib.vg_validate_motions_device(
        r, e, da.data_ptr(), db.data_ptr(), n, 32, o, bl, st))
    learned, learned_blocks = run(lambda r, e, o, bl, st: lib.vg_validate_motions_learned_device(
        r, e, m, da.data_ptr(), db.data_ptr(), n, 32, 16, o, bl, st))
    assert np.array_equal(learned, plain)
    assert np.array_equal(learned_blocks[plain == 1], plain_blocks[plain == 1])  # valid edges: every block
    coll = plain == 0
    assert learned_blocks[coll].sum() < plain_blocks[coll].sum(), (learned_blocks[coll].sum(), plain_blocks[coll].sum())
    assert np.all(learned_blocks[coll] >= 1)


@pytest.mark.parametrize("kind,lanes", [("random", 8), ("nan", 8), ("inf", 8), ("constant", 8), ("random", 4), ("constant", 4)])
def test_any_scores_keep_every_verdict(torch, kind, lanes):
    """The order is a permutation of each edge's blocks whatever the scores hold (8-lane blocks
    with the x86 bound, 4-lane blocks with the exact square root)."""
    from vamp_gb300 import scenes
    import vamp_gb300 as vg
    from vamp_gb300._lib import SQRT_EXACT, SQRT_X86, lib

    env = vg.Environment.from_scene(scenes.scene_config1(2), lanes=lanes, sqrt_mode=SQRT_X86 if lanes == 8 else SQRT_EXACT)
    a, b = scenes.edges(vg.panda.s_m, vg.panda.s_a, 8192, 31)
    n, probes = len(a), 32
    rng = np.random.default_rng(7)
    sc = rng.standard_normal((n, probes)).astype(np.float32)
    if kind == "nan":
        sc[rng.random(sc.shape) < 0.3] = np.nan
    elif kind == "inf":
        sc[rng.random(sc.shape) < 0.3] = np.inf
        sc[rng.random(sc.shape) < 0.3] = -np.inf
    elif kind == "constant":
        sc[:] = 1.0
    da, db, dsc = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), torch.from_numpy(sc).cuda()
    s = torch.cuda.current_stream().cuda_stream
    ref = torch.empty(n, dtype=torch.uint8, device="cuda")
    ref_blocks = torch.empty(n, dtype=torch.int32, device="cuda")
    env.set_schedule(1)
    assert lib.vg_validate_motions_device(b"panda", env.handle, da.data_ptr(), db.data_ptr(), n, 32, ref.data_ptr(),
                                          ref_blocks.data_ptr(), s) == 0
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    blocks = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = lib.vg_validate_motions_scored_device(b"panda", env.handle, da.data_ptr(), db.data_ptr(), n, 32, dsc.data_ptr(),
                                               probes, out.data_ptr(), blocks.data_ptr(), s)
    assert rc == 0, lib.vg_last_error()
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    valid = ref.bool()
    assert torch.equal(blocks[valid], ref_blocks[valid])
    if kind == "constant":  # ties keep the reference's order
        assert torch.equal(blocks, ref_blocks)
