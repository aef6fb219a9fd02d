"""GB300-native CVO / RKHS-BA registration core (drop-in for the CvoGPU path of UMich-CURLY/RKHS_BA).

The compute path is the native library built from ``rkhs_ba_gb300/csrc`` (CUDA for
sm_103a) and bound through its C ABI (``include/cvo_gb300.h``).
"""
import os

from .cloud import CvoPointCloud
from .cvo import AdaptiveCvoGPU, Association, CvoGPU, CvoParams, CvoResultInfo, GpuCloud

PARAMS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "params")


def params_path(name: str) -> str:
    """Path of a bundled parameter file (geometric, color, lidar_semantic, irls)."""
    return os.path.join(PARAMS_DIR, name + ".yaml")


__all__ = ["CvoPointCloud", "CvoGPU", "AdaptiveCvoGPU", "CvoParams", "CvoResultInfo", "Association", "GpuCloud", "params_path"]
