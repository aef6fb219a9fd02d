"""Generates the committed fixtures of tests/golden/ (run in a checkout where the
reference is mounted; the fixtures themselves travel with the repository).

demo_pair.npz   the reference's demo clouds demo_data/source.pcd (523 points) and
                demo_data/target.pcd (1080 points), xyz + colour features in the
                reference's (b, g, r) / 255 order, read with CvoPointCloud.read_pcd.
demo_oracle.npz oracle outputs on that pair (inner product at one lengthscale and a
                100-iteration registration with the colour parameters): a regression
                pin of the oracle.

usage: python tests/golden/make_golden.py [/path/to/reference]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from rkhs_ba_gb300 import CvoParams, CvoPointCloud, params_path  # noqa: E402


def main(ref_root="/root/reference"):
    src = CvoPointCloud.read_pcd(os.path.join(ref_root, "demo_data", "source.pcd"))
    tgt = CvoPointCloud.read_pcd(os.path.join(ref_root, "demo_data", "target.pcd"))
    np.savez_compressed(os.path.join(HERE, "demo_pair.npz"), src_xyz=src.xyz, src_feat=src.features,
                        tgt_xyz=tgt.xyz, tgt_feat=tgt.features)
    p = CvoParams(params_path("color"))
    p.MAX_ITER = 100
    ell = 0.4
    s = CvoPointCloud(src.xyz, src.features)
    t = CvoPointCloud(tgt.xyz, tgt.features)
    ip, z = orc.inner_product_gpu_semantics(p, s, t, np.eye(4), ell)
    ret, T, iters, _ = orc.align(p, s, t, np.eye(4))
    np.savez_compressed(os.path.join(HERE, "demo_oracle.npz"), ell=ell, ip=ip, ip_nnz=z, max_iter=p.MAX_ITER,
                        iters=iters, ret=ret, T_out=T)
    print("demo pair:", src.num_points(), tgt.num_points(), "ip", ip, z, "align", ret, iters)


if __name__ == "__main__":
    main(*sys.argv[1:])
