"""Gather-bandwidth calibration used as the sweep's access-pattern ceiling."""
import pytest

import gmr


@pytest.mark.gpu
def test_gather_bandwidth_l2_above_hbm():
    l2 = gmr.measure_gather_bandwidth(32 << 20)
    hbm = gmr.measure_gather_bandwidth(2 << 30)
    assert 500.0 < hbm < l2 < 50000.0
    seq = gmr.measure_gather_bandwidth(32 << 20, sequential=True)
    assert 0.5 * l2 < seq < 50000.0


def test_gather_bandwidth_rejects_bad_size():
    with pytest.raises(gmr.GmrError):
        gmr.measure_gather_bandwidth(16)
