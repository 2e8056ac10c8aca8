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


@pytest.mark.gpu
@pytest.mark.parametrize("mode,depth,unit", [("load16", 8, 128), ("load32", 4, 128), ("seq16", 16, 128),
                                             ("bulk", 8, 128), ("bulk", 2, 4096)])
def test_gather_load_paths(mode, depth, unit):
    """Every load path of the calibration runs to completion (bulk copies:
    every mbarrier wait completes) and gives a rate inside physical bounds."""
    gbs = gmr.measure_gather(32 << 20, mode=mode, depth=depth, unit_bytes=unit)
    assert 100.0 < gbs < 50000.0


@pytest.mark.parametrize("kw", [dict(mode="bulk", depth=66), dict(mode="bulk", depth=3), dict(mode="load16", depth=3),
                                dict(mode="load32", unit_bytes=16), dict(mode="bulk", depth=64, unit_bytes=4096),
                                dict(unit_bytes=96)])
def test_gather_rejects_bad_arguments(kw):
    """Checked on the host before any device work."""
    with pytest.raises(gmr.GmrError):
        gmr.measure_gather(32 << 20, **kw)
