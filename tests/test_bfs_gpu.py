"""GPU SpMSpV and BFS through the C ABI against the reference's golden
outputs and the oracle."""
import numpy as np
import pytest

from combblas_gb300 import bfs as B
from combblas_gb300 import generators as G
from conftest import golden_matrix

pytestmark = pytest.mark.gpu


def test_bfs_golden(gpu_ctx, golden):
    for name in ("seven_sym", "torus", "rmat8"):
        M = golden_matrix(golden, name).with_values(None)
        g = B.Graph(M)
        for s in golden[f"bfs/{name}/sources"]:
            par, lev, st = B.bfs(g, int(s))
            assert np.array_equal(par, golden[f"bfs/{name}/{s}/parents"]), (name, s)
            assert np.array_equal(lev, golden[f"bfs/{name}/{s}/levels"]), (name, s)
            assert st.iterations == int(golden[f"bfs/{name}/{s}/iters"]), (name, s)


@pytest.mark.parametrize("scale,ef", [(12, 16), (16, 16)])
def test_bfs_rmat_vs_oracle(gpu_ctx, oracle_lib, scale, ef):
    O = oracle_lib
    A = G.rmat(scale, ef, seed=scale, values=None)
    g = B.Graph(A)
    rng = np.random.default_rng(1)
    deg = np.diff(A.colptr)
    for s in rng.choice(np.nonzero(deg)[0], 4, replace=False):
        par, lev, st = B.bfs(g, int(s))
        epar, elev, eit = O.port_bfs(A, int(s))
        assert np.array_equal(par, epar) and np.array_equal(lev, elev)
        assert st.iterations == eit
        assert st.host_checks == 0  # the whole traversal ran as one graph (while node)
        reached = (par >= 0) | (np.arange(A.ncol) == s)
        assert st.reached == reached.sum()
        assert st.edges == deg[reached].sum() // 2


def test_bfs_device_graph_replay(gpu_ctx, oracle_lib):
    """The captured level graph, replayed for several sources into the same
    device buffers, gives the oracle's arrays each time."""
    import torch

    O = oracle_lib
    A = G.rmat(14, 8, seed=2, values=None)
    g = B.Graph(A)
    par = torch.empty(A.ncol, dtype=torch.int64, device="cuda")
    lev = torch.empty(A.ncol, dtype=torch.int64, device="cuda")
    for s in (0, 5, 77, 1000):
        B.bfs_device(g, s, par.data_ptr(), lev.data_ptr())
        epar, elev, _ = O.port_bfs(A, s)
        assert np.array_equal(par.cpu().numpy(), epar) and np.array_equal(lev.cpu().numpy(), elev)


def test_isolated_source(gpu_ctx):
    A = G.CSC(5, 5, np.array([0, 0, 1, 2, 2, 2]), np.array([2, 1]), None)
    par, lev, st = B.bfs(A, 0)
    assert (par == -1).all() and lev[0] == 0 and (lev[1:] == -1).all() and st.iterations == 1


def test_spmspv_golden(gpu_ctx, golden):
    M = golden_matrix(golden, "rmat8").with_values(None)
    g = B.Graph(M)
    yi, yv = B.SpMXSpV(g, golden["spmspv/rmat8/x_ind"], golden["spmspv/rmat8/x_val"])
    assert np.array_equal(yi, golden["spmspv/rmat8/y_ind"]) and np.array_equal(yv, golden["spmspv/rmat8/y_val"])


def test_spmspv_vs_oracle(gpu_ctx, oracle_lib):
    O = oracle_lib
    A = G.rmat(15, 8, seed=3, values=None)
    g = B.Graph(A)
    rng = np.random.default_rng(4)
    for nx in (0, 1, 100, 5000):
        x = np.sort(rng.choice(A.ncol, nx, replace=False)).astype(np.int32)
        xv = rng.integers(-10**12, 10**12, nx).astype(np.int64)
        yi, yv = B.SpMXSpV(g, x, xv)
        ei, ev = O.port_spmspv(A, x, xv)
        assert np.array_equal(yi, ei) and np.array_equal(yv, ev)


def test_spmspv_rejects_bad_index(gpu_ctx):
    from combblas_gb300._lib import GbcError

    A = G.rmat(8, 4, seed=1, values=None)
    g = B.Graph(A)
    with pytest.raises(GbcError):
        B.SpMXSpV(g, np.array([A.ncol + 5], np.int32), np.array([1], np.int64))


@pytest.mark.parametrize("policy", ["topdown", "bottomup", "auto"])
def test_bfs_directions_identical(gpu_ctx, oracle_lib, golden, policy):
    """Top-down, bottom-up and per-level switching give the reference's
    parents and levels (smallest frontier neighbour) bit for bit."""
    O = oracle_lib
    A = G.rmat(15, 16, seed=5, values=None)
    g = B.Graph(A)
    g.set_policy(policy)
    deg = np.diff(A.colptr)
    for s in np.random.default_rng(2).choice(np.nonzero(deg)[0], 5, replace=False):
        par, lev, st = B.bfs(g, int(s))
        epar, elev, eit = O.port_bfs(A, int(s))
        assert np.array_equal(par, epar) and np.array_equal(lev, elev) and st.iterations == eit
    for name in ("seven_sym", "torus", "rmat8"):
        M = golden_matrix(golden, name).with_values(None)
        gg = B.Graph(M)
        gg.set_policy(policy)
        for s in golden[f"bfs/{name}/sources"]:
            par, lev, st = B.bfs(gg, int(s))
            assert np.array_equal(par, golden[f"bfs/{name}/{s}/parents"]), (name, s, policy)
            assert np.array_equal(lev, golden[f"bfs/{name}/{s}/levels"]), (name, s, policy)
