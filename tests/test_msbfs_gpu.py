"""Multi-source BFS (the Select2ndMin SpGEMM loop of MD.cpp) on the GPU
against the reference's golden parents and the oracle's loop."""
import numpy as np
import pytest

from combblas_gb300 import bfs as B
from combblas_gb300 import generators as G
from conftest import golden_matrix

pytestmark = pytest.mark.gpu


def test_msbfs_golden(gpu_ctx, golden):
    for name in ("rmat8", "torus"):
        M = golden_matrix(golden, name).with_values(None)
        g = B.Graph(M)
        par, st = B.msbfs(g, golden[f"msbfs/{name}/roots"])
        assert np.array_equal(par, golden[f"msbfs/{name}/parents"]), name
        g.close()


@pytest.mark.parametrize("scale,ef,nroots", [(11, 8, 64), (13, 16, 128)])
def test_msbfs_rmat_vs_oracle(gpu_ctx, oracle_lib, scale, ef, nroots):
    O = oracle_lib
    A = G.rmat(scale, ef, seed=scale + 3, values=None)
    deg = np.diff(A.colptr)
    roots = np.random.default_rng(5).choice(np.nonzero(deg)[0], nroots, replace=False)
    roots[1] = roots[0]  # a repeated root is just another tree
    g = B.Graph(A)
    par, st = B.msbfs(g, roots)
    ref, levels = O.port_msbfs(A, roots)
    assert np.array_equal(par, ref)
    assert st.host_checks == 0  # every level on the device, one graph launch
    reached = par >= 0
    assert st.reached == int(reached.sum())
    assert st.edges == int((reached * deg[None, :]).sum()) // 2
    assert st.levels == levels
    # again (state reset between calls), and into a device buffer
    import torch

    dp = torch.empty((len(roots), A.ncol), dtype=torch.int64, device="cuda")
    _, st2 = B.msbfs(g, roots, dp.data_ptr())
    assert np.array_equal(dp.cpu().numpy(), ref) and st2.reached == st.reached
    g.close()


def test_msbfs_isolated_and_errors(gpu_ctx):
    from combblas_gb300._lib import GbcError

    A = G.rmat(9, 4, seed=2, values=None)
    deg = np.diff(A.colptr)
    iso = int(np.nonzero(deg == 0)[0][0])
    g = B.Graph(A)
    par, st = B.msbfs(g, [iso])
    assert par[0, iso] == iso and (par[0] >= 0).sum() == 1 and st.reached == 1
    with pytest.raises(GbcError, match="root out of range"):
        B.msbfs(g, [A.ncol])
    g.close()
