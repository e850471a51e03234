"""The learned form: the rank predictor's kernels against a CPU restatement, its training on the
plain recompression's own records, the sketch recompression against the oracle, and what the
trained network gains over sizing the sketch without it.

Bars: GPU gradients and predictions within 1e-3 (relative to the largest entry) of the float64
restatement with the same BF16 weights (FP32 accumulation and erff on the GPU); a learned
multiply's tiles within 2 x max(oracle's error, accuracy) of the exact product with every new
rank within +-1 of the oracle's; the trained predictor's mean absolute log2-rank error below
that of the input-rank rule it replaces.
"""
import numpy as np
import pytest

from oracle import hcore_oracle as O
from oracle import rank_mlp as R
from tests.helpers import load_tile_matrix, oracle_tile_grid, rel_fro

pytestmark = pytest.mark.gpu

ACC = 1e-8


@pytest.fixture(scope="module")
def env():
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import rank_model as RM
    from hcorepp_gb300 import tiles as T
    assert torch.cuda.is_available()
    return torch, L, T, RM


def test_mlp_forward_and_gradient_match_cpu_restatement(env):
    torch, L, T, RM = env
    rng = np.random.default_rng(3)
    m = RM.RankModel(seed=11)
    p = m.params()
    X = rng.uniform(-1.5, 1.5, size=(300, R.F)).astype(np.float32)
    t = rng.uniform(0.0, 7.0, size=300).astype(np.float32)
    xd, td = torch.from_numpy(X).cuda(), torch.from_numpy(t).cuda()
    y_gpu = m.predict(xd).cpu().numpy()
    y_cpu, _ = R.forward(p, X.astype(np.float64))
    assert np.abs(y_gpu - y_cpu).max() <= 1e-3 * max(1.0, np.abs(y_cpu).max())
    g_gpu, loss_gpu = m.gradient(xd, td)
    g_cpu, loss_cpu = R.gradient(p, X.astype(np.float64), t.astype(np.float64))
    assert abs(loss_gpu - loss_cpu) <= 1e-3 * loss_cpu
    scale = np.abs(g_cpu).max()
    assert np.abs(g_gpu - g_cpu).max() <= 1e-3 * scale, (np.abs(g_gpu - g_cpu).max(), scale)
    # every parameter block receives gradient
    o = 0
    for name, shape in R.SIZES:
        n = int(np.prod(shape))
        assert np.abs(g_gpu[o:o + n]).max() > 0, name
        o += n
    m.close()


def _problem(env, seed, n=2048, nb=256):
    torch, L, T, RM = env
    from hcorepp_gb300.problems import KernelMatrix
    nt = n // nb
    ka = KernelMatrix(n, nb, 2, 0.1, seed)
    kc = KernelMatrix(n, nb, 2, 0.1, seed + 1)
    ga = oracle_tile_grid(ka, nt, ACC, True)
    gc = oracle_tile_grid(kc, nt, ACC, True)
    return ga, gc, nt, nb


def _harvest(env, seeds):
    torch, L, T, RM = env
    feats, infos = [], []
    params = T.CompressionParameters(ACC, truncated_svd=True)
    for s in seeds:
        ga, gc, nt, nb = _problem(env, s)
        A = load_tile_matrix(T, L, ga, nb, nb // 3)
        Cm = load_tile_matrix(T, L, gc, nb, nb // 3)
        f, i = RM.harvest_multiply(A, A, Cm, params)
        feats.append(f)
        infos.append(i)
    return torch.cat(feats), torch.cat(infos)


@pytest.fixture(scope="module")
def trained(env):
    torch, L, T, RM = env
    RM.learned_off()
    feats, info = _harvest(env, seeds=(3, 5, 7, 9))
    m = RM.RankModel(seed=5)
    loss0, used = m.train(feats, info, epochs=1, batch=128, lr=1e-3)
    loss, used = m.train(feats, info, epochs=60, batch=128, lr=2e-3)
    return m, loss0, loss, used


def test_training_on_plain_records_reduces_the_loss(env, trained):
    m, loss0, loss, used = trained
    assert used > 1000
    assert loss < 0.25 * loss0, (loss0, loss)
    assert loss < 0.1  # mean squared log2-rank error: ranks predicted within ~25 %


def test_trained_predictor_beats_the_input_rank_rule(env, trained):
    torch, L, T, RM = env
    m = trained[0]
    RM.learned_off()
    feats, info = _harvest(env, seeds=(21,))  # held-out inputs
    rec = info.cpu().numpy()
    keep = (rec[:, 4] > 0) & (rec[:, 0] == 0)
    true = np.log2(1.0 + rec[keep, 5])
    pred = m.predict(feats).cpu().numpy()[keep]
    ra, rb, rc = rec[keep, 1], rec[keep, 2], rec[keep, 3]
    add = np.where((ra > 0) & (rb > 0), np.minimum(ra, rb), np.maximum(ra, rb))
    rule = np.log2(1.0 + np.maximum(rc, add))
    err_net, err_rule = np.abs(pred - true).mean(), np.abs(rule - true).mean()
    print(f"mean |log2 rank error|: network {err_net:.3f}, input-rank rule {err_rule:.3f}")
    assert err_net < err_rule


@pytest.mark.parametrize("policy", [0, 1])
def test_learned_multiply_vs_oracle(env, trained, policy):
    torch, L, T, RM = env
    m = trained[0]
    ga, gc, nt, nb = _problem(env, 13)
    A = load_tile_matrix(T, L, ga, nb, nb // 3)
    Cm = load_tile_matrix(T, L, gc, nb, nb // 3)
    exact = A.to_dense() @ A.to_dense() + Cm.to_dense()
    if policy == 0:
        m.enable()
    else:
        RM.learned_without_network()
    info = T.info_buffer(nt ** 3)
    ctx = T.run_context()
    ctx.set_sketch_limit(100)  # every update whose sketch is narrower than its stacks: the sketch path under test
    try:
        T.tlr_gemm(1.0, A, A, 1.0, Cm, T.CompressionParameters(ACC, truncated_svd=True), info)
        torch.cuda.synchronize()
    finally:
        RM.learned_off()
        ctx.set_sketch_limit(0)
    rec = info.cpu().numpy()
    assert int(rec[:, 0].max()) == 0
    sketched = int(np.count_nonzero(rec[:, 13] > 0))
    accepted = int(np.count_nonzero(rec[:, 14] > 0))
    print(f"policy {policy}: {sketched} sketched, {accepted} accepted of {int(np.count_nonzero(rec[:, 4] > 0))}")
    assert sketched > 0
    O.tile_matrix_multiply(ga, ga, gc, 1.0, 1.0, O.CompressionParameters(ACC, truncated_svd=True))
    g = Cm.to_dense()
    ranks = Cm.rank_grid()
    for i in range(nt):
        for j in range(nt):
            sl = (slice(i * nb, (i + 1) * nb), slice(j * nb, (j + 1) * nb))
            e_o = rel_fro(gc[i][j].to_dense(), exact[sl])
            assert rel_fro(g[sl], exact[sl]) <= 2 * max(e_o, ACC), (i, j)
            if gc[i][j].kind != "dense":
                assert abs(int(ranks[i, j]) - gc[i][j].rank) <= 1, (i, j, ranks[i, j], gc[i][j].rank)


def test_default_sketch_limit_keeps_sketches_to_half_the_stack(env, trained):
    """hcgb_set_sketch_limit: by default an update is sketched only when its sketch (with the probe
    columns) is at most half its stack width; the result keeps the same accuracy bar."""
    torch, L, T, RM = env
    m = trained[0]
    ga, gc, nt, nb = _problem(env, 13)
    A = load_tile_matrix(T, L, ga, nb, nb // 3)
    Cm = load_tile_matrix(T, L, gc, nb, nb // 3)
    exact = A.to_dense() @ A.to_dense() + Cm.to_dense()
    m.enable()
    info = T.info_buffer(nt ** 3)
    try:
        T.tlr_gemm(1.0, A, A, 1.0, Cm, T.CompressionParameters(ACC, truncated_svd=True), info)
        torch.cuda.synchronize()
    finally:
        RM.learned_off()
    rec = info.cpu().numpy()
    assert int(rec[:, 0].max()) == 0
    sk = rec[:, 13] > 0
    assert np.all(2 * (rec[sk, 13] + 4) <= rec[sk, 4]), rec[sk][:, [4, 13]]
    O.tile_matrix_multiply(ga, ga, gc, 1.0, 1.0, O.CompressionParameters(ACC, truncated_svd=True))
    o = np.block([[t.to_dense() for t in row] for row in gc])
    assert rel_fro(Cm.to_dense(), exact) <= 2 * max(rel_fro(o, exact), ACC)
