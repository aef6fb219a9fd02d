"""Parity at the configured full sizes, through the C ABI.

Whole kernel matrices against the oracle (which finishes these in seconds: it prunes
with a grid and runs on all host threads):

* 10,000-point geometric room pair (geometric.yaml, lengthscale 0.25);
* 50,000-point colour stereo pair (color.yaml, lengthscale 0.4, identity pose): about
  5 M kept pairs, 20 k rows above the 256-pair cap, so the index-ordered selection
  (k_select / k_rescan) runs on tens of thousands of rows;
* 128,000-point semantic LiDAR scan pair (lidar_semantic.yaml, 19 classes,
  lengthscale 1.0).

Column sets bit-exact and values within 1e-5 relative (the bar of the smaller parity
cases), and the GPU inner product equal to the oracle's within 1e-5 relative.  The
library reads the parameter file with its own reader and the oracle with its own
(oracle/params.py), so the two sides share no parser.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle.params import OracleParams
from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes

pytestmark = pytest.mark.gpu

REL = 1e-5


def _ell_to_csr(ind, val, nnz):
    """Oracle ELL (rows of cap slots, nnz used) as CSR arrays in row order."""
    cap = ind.shape[1]
    used = np.arange(cap)[None, :] < nnz[:, None]
    row_ptr = np.concatenate([[0], np.cumsum(nnz, dtype=np.int64)])
    return row_ptr, ind[used], val[used]


def _check(name, src, tgt, T, ell):
    cvo = CvoGPU(params=CvoParams(params_path(name)))
    oparams = OracleParams(params_path(name))
    a = cvo.compute_association_gpu(src, tgt, T, ell)
    ind, val, nnz = orc.association(oparams, src, tgt, T, ell)
    row_ptr, col, v = _ell_to_csr(ind, val, nnz)
    assert a.rows == src.num_points()
    assert np.array_equal(np.asarray(a.row_ptr, np.int64), row_ptr)
    assert np.array_equal(np.asarray(a.col), col)
    gv = np.asarray(a.val, np.float64)
    ov = v.astype(np.float64)
    bad = np.abs(gv - ov) > REL * np.abs(ov)
    assert not bad.any(), (int(bad.sum()), np.nonzero(bad)[0][:5])
    g = cvo.inner_product_gpu(src, tgt, T, ell)
    o, _ = orc.inner_product_gpu_semantics(oparams, src, tgt, T, ell)
    assert g == pytest.approx(o, rel=REL)
    return nnz


def test_full_size_geometric_10k(cuda_device):
    src, tgt, _ = scenes.room_pair(n=10000, seed=1)
    nnz = _check("geometric", src, tgt, np.eye(4, dtype=np.float32), 0.25)
    assert nnz.sum() > 50000


def test_full_size_colour_50k(cuda_device):
    src, tgt, _ = scenes.stereo_pair(n=50000, seed=2)
    nnz = _check("color", src, tgt, np.eye(4, dtype=np.float32), 0.4)
    assert nnz.sum() > 4_000_000
    cap = OracleParams(params_path("color")).nearest_neighbors_max
    assert (nnz == cap).sum() > 10000          # the capped-row selection ran


def test_full_size_semantic_lidar_128k(cuda_device):
    src, tgt, _ = scenes.lidar_pair(n=128000, seed=1)
    nnz = _check("lidar_semantic", src, tgt, np.eye(4, dtype=np.float32), 1.0)
    assert nnz.sum() > 1_000_000
