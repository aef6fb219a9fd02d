"""The autotuner's configuration store (cvo_tune_set / cvo_tune_get) on the host: one
entry per (features, classes, floor(log2 rows)) key, defaults (4, 8) for untuned keys,
invalid divisors rejected.  No GPU needed."""
import numpy as np
import pytest

from rkhs_ba_gb300 import CvoGPU, CvoParams
from rkhs_ba_gb300._lib import CvoError


@pytest.fixture()
def cvo():
    return CvoGPU(params=CvoParams())


def test_untuned_keys_report_the_default(cvo):
    assert cvo.tune_get(5, 0, 50000) == (4.0, 8.0, False)


def test_rows_share_a_key_within_one_power_of_two(cvo):
    cvo.tune_set(5, 0, 50000, 6.0, 4.0)
    for rows in (32768, 40000, 50000, 65535):
        assert cvo.tune_get(5, 0, rows) == (6.0, 4.0, True), rows
    for rows in (32767, 65536, 128000):
        assert cvo.tune_get(5, 0, rows)[2] is False, rows
    # the feature and class counts are part of the key
    assert cvo.tune_get(3, 0, 50000)[2] is False
    assert cvo.tune_get(5, 19, 50000)[2] is False


def test_a_later_setting_replaces_the_entry(cvo):
    cvo.tune_set(1, 19, 128000, 2.0, 16.0)
    cvo.tune_set(1, 19, 100000, 3.0, 8.0)              # same key (2^16 <= rows < 2^17)
    assert cvo.tune_get(1, 19, 128000) == (3.0, 8.0, True)


@pytest.mark.parametrize("div_r, div_ext", [(0.0, 8.0), (4.0, 0.0), (-1.0, 8.0), (float("nan"), 8.0)])
def test_invalid_divisors_are_rejected(cvo, div_r, div_ext):
    with pytest.raises(CvoError):
        cvo.tune_set(5, 0, 50000, div_r, div_ext)
    assert cvo.tune_get(5, 0, 50000)[2] is False


def test_negative_sizes_are_rejected(cvo):
    with pytest.raises(CvoError):
        cvo.tune_set(-1, 0, 1000, 4.0, 8.0)
    with pytest.raises(CvoError):
        cvo.tune_set(5, 0, -5, 4.0, 8.0)
