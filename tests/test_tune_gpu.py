"""GPU tests of the autotuner: every layout and SpMM column tile it can choose gives
the oracle's results (bit-exact on rows folded in storage order, rtol 1e-5 against
FP64 elsewhere), and the chosen configuration sticks to the handle."""
import numpy as np
import pytest
import torch

import gpugraphs as G
from gpugraphs import generators as gen
from gpugraphs import tuning
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def rmat14():
    A = gen.rmat(14, 16, seed=51, wkind=gen.W_U01_F32)
    rp, cv, nz = host(A.rowptr), host(A.colval), host(A.nzval)
    x = np.random.default_rng(51).random(A.n, dtype=np.float32)
    return A, rp, cv, nz, x


def spmv_check(A, rp, cv, nz, x):
    m = A.m
    y = torch.zeros(m, dtype=torch.float32, device="cuda")
    G.gpu_spmv_(y, A, torch.from_numpy(x).cuda())
    yh = host(y)
    yo = np.zeros(m, np.float32)
    O.csr_spmv(m, A.n, rp, cv, nz, yo, x)
    short = np.diff(rp) <= 32
    assert (yh[short] == yo[short]).all()
    ref64 = np.zeros(m)
    rows = np.repeat(np.arange(m), np.diff(rp))
    np.add.at(ref64, rows, nz.astype(np.float64) * x[cv - 1].astype(np.float64))
    np.testing.assert_allclose(yh, ref64, rtol=RTOL, atol=1e-6)


@pytest.mark.parametrize("choice", [
    {"spmv_kernel": "csr_row_blocks", "block_rows": 32},
    {"spmv_kernel": "csr_row_blocks", "block_rows": 128},
    {"spmv_kernel": "sell", "slice_size": 8, "sigma": 64},
    {"spmv_kernel": "sell", "slice_size": 16, "sigma": 1024},
    {"spmv_kernel": "sell", "slice_size": 32, "sigma": 16384},
    {"spmv_kernel": "window_tiles"},
])
def test_every_spmv_layout_matches_oracle(rmat14, choice):
    A, rp, cv, nz, x = rmat14
    tuning.apply(A, choice)
    spmv_check(A, rp, cv, nz, x)


@pytest.mark.parametrize("tile", [32, 64, 128])
def test_every_spmm_tile_matches_oracle(rmat14, tile):
    A, rp, cv, nz, _ = rmat14
    k = 160
    tuning.apply(A, {"spmm_column_tile": tile})
    B = np.random.default_rng(tile).random((A.n, k), dtype=np.float32)
    Cd = torch.zeros((A.m, k), dtype=torch.float32, device="cuda")
    G.gpu_spmm_(Cd, A, torch.from_numpy(B).cuda())
    Ch = host(Cd)
    Co = np.zeros((A.m, k), np.float32)
    O.csr_spmm(A.m, rp, cv, nz, Co, B, layout=1)
    short = np.diff(rp) <= 256
    assert (Ch[short] == Co[short]).all()
    np.testing.assert_allclose(Ch, Co, rtol=1e-4, atol=1e-4)


def test_autotune_picks_and_keeps_a_choice(rmat14):
    A, rp, cv, nz, x = rmat14
    res = G.autotune(A, spmm_k=64)
    assert res["spmv_kernel"] in ("csr_row_blocks", "sell", "window_tiles")
    assert res["candidates"] >= 6
    assert res["spmv_ms"] <= res["spmv_default_ms"] * 1.0001
    assert res["spmm_column_tile"] in (32, 64)
    spmv_check(A, rp, cv, nz, x)
    B = gen.rmat(14, 16, seed=51, wkind=gen.W_U01_F32)  # same matrix, new handle
    res2 = tuning.autotune_cached(A, 64)
    res3 = tuning.autotune_cached(B, 64)
    assert res3["cached"] and res3["spmv_kernel"] == res2["spmv_kernel"]
    spmv_check(B, rp, cv, nz, x)


def test_autotune_rejects_non_float32():
    A = gen.rmat(10, 8, seed=52, wkind=gen.W_INT_1_255)
    with pytest.raises(G.UnsupportedError):
        G.autotune(A)
