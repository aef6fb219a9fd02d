"""Host cloud container edge cases (CvoPointCloud, include/UnifiedCvo/utils/CvoPointCloud.hpp:32-221)."""
import numpy as np

from rkhs_ba_gb300 import CvoPointCloud


def test_empty_cloud_keeps_its_dimensions():
    c = CvoPointCloud(np.zeros((0, 3), np.float32), np.zeros((0, 5), np.float32), np.zeros((0, 19), np.float32))
    assert c.num_points() == 0 and c.feature_dimensions() == 5 and c.num_classes() == 19
    cs = c.c_struct()
    assert cs.n == 0 and cs.F == 5 and cs.C == 19


def test_flat_feature_arrays_are_reshaped_per_point():
    c = CvoPointCloud(np.ones((4, 3)), np.arange(20, dtype=np.float32))
    assert c.features.shape == (4, 5) and c.features.dtype == np.float32
    assert np.array_equal(c.features[1], np.arange(5, 10, dtype=np.float32))
