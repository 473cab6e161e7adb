"""Workload definitions of bench.py that need no GPU: the AdResS workload
scaled to another molecule count keeps its density and slab proportions."""
import numpy as np


def test_adress_config_default_is_the_workload():
    import bench

    assert bench.adress_config() == bench.ADRESS
    assert bench.adress_config(bench.ADRESS["n"]) == bench.ADRESS


def test_adress_config_scaled_keeps_density_and_proportions():
    import bench

    a = bench.ADRESS
    c = bench.adress_config(4_000_000)
    assert c["n"] == 4_000_000
    rho = lambda d: d["n"] / np.prod(d["box"])
    assert abs(rho(c) - rho(a)) <= 1e-12 * rho(a)
    f = c["box"][0] / a["box"][0]
    np.testing.assert_allclose(np.asarray(c["box"]) / np.asarray(a["box"]), f, rtol=1e-12)
    np.testing.assert_allclose(np.asarray(c["center"]) / np.asarray(a["center"]), f, rtol=1e-12)
    assert abs(c["at"] / a["at"] - f) <= 1e-12 * f
    # the hybrid width, bin width and physics stay those of the workload
    for k in ("hy", "binw", "rc", "skin", "cap", "dt", "T", "gamma", "K"):
        assert c[k] == a[k]
    pos, vel = bench.adress_initial(0, bench.adress_config(50_000))
    assert pos.shape == (50_000, 3) and vel.shape == (50_000, 3)
    assert (pos >= 0).all() and (pos < np.asarray(bench.adress_config(50_000)["box"])).all()
