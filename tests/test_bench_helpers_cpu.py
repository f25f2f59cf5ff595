"""bench.py's roofline arithmetic on the CPU (no GPU)."""
import pytest

import bench


def test_fp64_order_bound_of_the_256_laplacian():
    # 17 FP64 instructions per point at 1.68 per clock per SM on 152 SMs at
    # 2070 MHz: 31.1 G points/s; 16.38 algorithmic bytes per interior point
    # (262,144,512 B over 252^3 points) make that 509 GB/s
    bpp = 262144512 / 252 ** 3
    fb = bench.fp64_order_bound(931.0, bpp)
    assert fb["gbs"] == pytest.approx(1.68 * 152 * 2070e6 / 17 * bpp / 1e9)
    assert 500 < fb["gbs"] < 520
    assert fb["frac"] == pytest.approx(931.0 / fb["gbs"])
    assert fb["fp64_per_point"] == 17
    # a slower clock lowers the bound in proportion
    assert bench.fp64_order_bound(931.0, bpp, sm_mhz=1035.0)["gbs"] == pytest.approx(fb["gbs"] / 2)
