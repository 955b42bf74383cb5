"""Learned output sizing on the GPU: the training kernels against the
float64 oracle, and learned products bit-identical to the exact two-phase
path (including forced overflow)."""
import numpy as np
import pytest

from combblas_gb300 import generators as G
from combblas_gb300 import local, mcl, sizing
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def test_gradient_kernels_match_oracle(gpu_ctx):
    rng = np.random.default_rng(1)
    m = sizing.SizingModel(seed=7)
    p, _ = m.get()
    feat = rng.normal(0, 1, (777, 6)).astype(np.float32)
    target = rng.normal(0, 1, 777).astype(np.float32)
    g = m.gradient(feat, target)[:mlp_ref.NP + 1]
    ref = mlp_ref.gradient(p.astype(np.float64), feat.astype(np.float64), target.astype(np.float64))
    rel = np.linalg.norm(g[:mlp_ref.NP] - ref[:mlp_ref.NP]) / np.linalg.norm(ref[:mlp_ref.NP])
    assert rel < 1e-5, rel
    assert abs(g[mlp_ref.NP] - ref[mlp_ref.NP]) <= 1e-5 * ref[mlp_ref.NP]
    pred = m.predict(feat)
    assert np.allclose(pred, mlp_ref.predict(p.astype(np.float64), feat), rtol=1e-4, atol=1e-4)
    m.close()


def trained_model(A, seed=0):
    feat, flop, nnz = sizing.features(A, A)
    m = sizing.SizingModel(seed=seed)
    info = m.fit(feat, nnz, steps=300)
    return m, info, feat, flop, nnz


def test_training_reduces_loss_and_is_deterministic(gpu_ctx):
    A = G.rmat(13, 8, seed=31)
    feat, flop, nnz = sizing.features(A, A)
    nz = nnz > 0
    t = np.log2(1 + nnz[nz]).astype(np.float32)
    losses = []
    for _ in range(2):
        m = sizing.SizingModel(seed=3)
        l0 = m.train(feat[nz], t, steps=0)
        l1 = m.train(feat[nz], t, steps=300)
        losses.append((l0, l1, m.get()[0].copy()))
        m.close()
    assert losses[0][1] < 0.2 * losses[0][0]
    assert np.array_equal(losses[0][2], losses[1][2])  # bit-identical training runs


@pytest.mark.parametrize("kind", ["rmat", "mcl"])
def test_learned_identical_to_exact(gpu_ctx, kind):
    # the model is trained on another matrix of the same statistics class
    if kind == "rmat":
        A = G.rmat(14, 8, seed=41)
        Atrain = G.rmat(14, 8, seed=42)
        dt = np.float64
    else:
        A = G.mcl_planted(1 << 15, 512, 20, 5, seed=43)
        Atrain = G.mcl_planted(1 << 15, 512, 20, 5, seed=44)
        dt = np.float32
    m, info, _, _, _ = trained_model(Atrain)
    m.use()
    Re = local.spgemm(A, A, dtype=dt)
    Rl = local.spgemm(A, A, dtype=dt, sizing="learned")
    ce, cl = Re.to_csc(), Rl.to_csc()
    assert all(np.array_equal(x, y) for x, y in zip(ce, cl))
    st = Rl.stats
    assert st.overflow_cols <= 0.05 * A.ncol
    m.close()


def test_forced_overflow_reruns_exactly(gpu_ctx):
    A = G.rmat(12, 8, seed=51)
    m, _, _, _, _ = trained_model(A)
    m.set_margin(-20.0)  # every capacity clamps to 1: (nearly) every column overflows
    m.use()
    Re = local.spgemm(A, A)
    Rl = local.spgemm(A, A, sizing="learned")
    assert all(np.array_equal(x, y) for x, y in zip(Re.to_csc(), Rl.to_csc()))
    nonempty = int((np.diff(Re.to_csc()[0]) > 1).sum())
    assert Rl.stats.overflow_cols >= nonempty
    m.close()


def test_model_beats_flop_bound_sizing(gpu_ctx):
    """What the network gains over sizing without it: the capacity it
    allocates is far below the multiplication-count bound (the only size
    known without a symbolic pass), at a small overflow rate."""
    A = G.rmat(15, 8, seed=61)
    m, info, feat, flop, nnz = trained_model(G.rmat(15, 8, seed=62))
    m.use()
    Rl = local.spgemm(A, A, sizing="learned")
    st = Rl.stats
    bound = int(np.minimum(sizing.features(A, A, exact=False)[1], A.nrow).sum())
    assert st.alloc_entries < 0.6 * bound
    assert st.overflow_cols < 0.02 * A.ncol
    m.close()


def test_mcl_learned_identical(gpu_ctx):
    A = G.mcl_planted(1 << 15, 512, 24, 6, seed=71)
    m, _, _, _, _ = trained_model(G.mcl_planted(1 << 15, 512, 24, 6, seed=72))
    m.use()
    Re, se = mcl.mcl_expand(A, 1e-4, 50, sizing="exact")
    Rl, sl = mcl.mcl_expand(A, 1e-4, 50, sizing="learned")
    assert all(np.array_equal(x, y) for x, y in zip(Re.to_csc(), Rl.to_csc()))
    m.close()


def test_model_persistence(gpu_ctx, tmp_path):
    A = G.rmat(12, 8, seed=81)
    m, _, feat, _, _ = trained_model(A)
    path = str(tmp_path / "sizing.json")
    m.save(path, sizing.stats_class(A))
    m2 = sizing.SizingModel(seed=99)
    assert m2.load(path, sizing.stats_class(A))
    assert np.array_equal(m.predict(feat), m2.predict(feat))
    assert m.get()[1] == m2.get()[1]
    m.close()
    m2.close()
