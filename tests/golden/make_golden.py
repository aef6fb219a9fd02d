"""Generates the committed fixtures of tests/golden/ from a checkout of the reference
(UMich-CURLY/RKHS_BA); the fixtures themselves travel with the repository, so no test
reads the reference at run time.

demo_pair.npz            the reference's demo clouds demo_data/source.pcd (523 points) and
                         demo_data/target.pcd (1080 points), xyz + colour features in the
                         reference's (b, g, r) / 255 order, read with CvoPointCloud.read_pcd.
demo_oracle.npz          oracle outputs on that pair (inner product at one lengthscale, a
                         10-iteration and a 100-iteration registration with the colour
                         parameters, read by the oracle's own yaml reader): a regression pin
                         of the oracle and the reference-data case of the GPU parity tests.
icosahedral_rotations.npz
                         the 60 rotation matrices gen_icosahedron_init_rots lists
                         (src/cvo/CvoGPU.cpp:279-342), parsed from the reference source as
                         data: the golden set the library's regenerated grid is checked against.

usage: python tests/golden/make_golden.py <reference checkout>
       (or set RKHS_BA_REFERENCE to the checkout's root)
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from oracle.params import OracleParams  # noqa: E402
from rkhs_ba_gb300 import CvoPointCloud, params_path  # noqa: E402


def icosahedral_rotations(ref_root):
    """The `pose[k] << r00, r01, ...;` rows of gen_icosahedron_init_rots as (60, 3, 3)."""
    with open(os.path.join(ref_root, "src", "cvo", "CvoGPU.cpp")) as fh:
        txt = fh.read()
    mats = [np.array([float(v) for v in m.group(1).split(",")]).reshape(3, 3)
            for m in re.finditer(r"pose\[\d+\]<<([^;]+);", txt)]
    if len(mats) != 60:
        raise RuntimeError("expected 60 rotations, found %d" % len(mats))
    return np.stack(mats)


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("RKHS_BA_REFERENCE")
    if not ref_root:
        sys.exit(__doc__)
    src = CvoPointCloud.read_pcd(os.path.join(ref_root, "demo_data", "source.pcd"))
    tgt = CvoPointCloud.read_pcd(os.path.join(ref_root, "demo_data", "target.pcd"))
    np.savez_compressed(os.path.join(HERE, "demo_pair.npz"), src_xyz=src.xyz, src_feat=src.features,
                        tgt_xyz=tgt.xyz, tgt_feat=tgt.features)
    p = OracleParams(params_path("color"))
    p.MAX_ITER = 100
    ell = 0.4
    s = CvoPointCloud(src.xyz, src.features)
    t = CvoPointCloud(tgt.xyz, tgt.features)
    ip, z = orc.inner_product_gpu_semantics(p, s, t, np.eye(4), ell)
    ret, T, iters, _ = orc.align(p, s, t, np.eye(4))
    q = p.copy()
    q.MAX_ITER = 10
    ret10, T10, iters10, _ = orc.align(q, s, t, np.eye(4))
    np.savez_compressed(os.path.join(HERE, "demo_oracle.npz"), ell=ell, ip=ip, ip_nnz=z, max_iter=p.MAX_ITER,
                        iters=iters, ret=ret, T_out=T, ret10=ret10, iters10=iters10, T_out10=T10)
    np.savez_compressed(os.path.join(HERE, "icosahedral_rotations.npz"), R=icosahedral_rotations(ref_root))
    print("demo pair:", src.num_points(), tgt.num_points(), "ip", ip, z, "align", ret, iters)


if __name__ == "__main__":
    main(*sys.argv[1:])
