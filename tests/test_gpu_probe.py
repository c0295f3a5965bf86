"""The read-bandwidth probe (bvhgpu_read_bandwidth) that gives the L2
ceiling reported beside the HBM roofline: a buffer that fits L2 reads faster
than one far larger than L2, and both rates are plausible for a GB300."""
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402

pytestmark = pytest.mark.gpu


def test_l2_reads_faster_than_hbm():
    l2 = pkg.read_bandwidth(60 << 20, passes=10, repeats=3)
    hbm = pkg.read_bandwidth(2 << 30, passes=1, repeats=3)
    assert 1000.0 < hbm < 12000.0
    assert l2 > hbm
