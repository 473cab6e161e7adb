"""Thermodynamic-force table text: io::dumpThermoForce / io::restoreThermoForce.

The known-answer case is io/ThermoForce.test.cpp:11-112 of the reference:
subdomain x in [1, 4], 100 bins, force(bin, type) = (bin + 1)(type + 1),
one and five types, dumped and restored, grid and forces compared with
EXPECT_FLOAT_EQ (4 float ulps).  The text itself is compared byte for byte
with the oracle's restatement of DumpProfile::dumpScalarView.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _lib_io():
    from mrmd_gb300 import io
    return io


def _kat(num_types, num_bins=100):
    grid = O.tf_grid(1.0, 4.0, num_bins)
    i = np.arange(num_bins, dtype=np.float64)[:, None]
    j = np.arange(num_types, dtype=np.float64)[None, :]
    return grid, (i + 1.0) * (j + 1.0)


def _float_eq(a, b):
    np.testing.assert_array_max_ulp(np.float32(a), np.float32(b), maxulp=4)


# ------------------------------------------------------------- oracle pin --

@pytest.mark.parametrize("num_types", [1, 5])
def test_oracle_kat_round_trip(num_types):
    """ThermoForce.test.cpp dumpSingleForce / dumpMultipleForces through the oracle:
    restoring the text gives the same grid (re-derived from the file's bin width,
    as the reference's constructor does) and forces."""
    grid, force = _kat(num_types)
    text = O.tf_table_text(grid, force, 0 if num_types == 1 else None)
    g2, f2, bw = O.tf_table_parse(text)
    sd = O.subdomain([1, 2, 3], [4, 6, 8], 0.5)
    nb = O.tf_num_bins(sd, bw)
    assert nb == 100
    _float_eq(O.tf_grid(1.0, 4.0, nb), grid)
    _float_eq(g2, grid)
    _float_eq(f2, force)


def test_oracle_text_layout():
    text = O.tf_table_text([0.5, 1.5], [[1.0, -2.0], [3.25, 1e-7]])
    assert text == "0.5 1.5\n1 3.25\n-2 1e-07\n"
    assert O.tf_table_text([0.5, 1.5], [[1.0, -2.0], [3.25, 1e-7]], 1) == "0.5 1.5\n-2 1e-07\n"
    # 6 significant digits, exponent form beyond them
    assert O.tf_table_text([0.123456789, 1234567.0], [[0.0], [-0.0]]) == "0.123457 1.23457e+06\n0 -0\n"


# ------------------------------------------------------- library (host) ----

@pytest.mark.parametrize("type_id", [None, 0, 3])
def test_write_table_text_matches_oracle(tmp_path, type_id):
    io = _lib_io()
    grid, force = _kat(5)
    p = tmp_path / "tf.txt"
    io.write_table(p, grid, force, type_id)
    assert p.read_text() == O.tf_table_text(grid, force, type_id)


def test_write_table_random_values_match_oracle(tmp_path):
    io = _lib_io()
    rng = np.random.default_rng(7)
    grid = np.sort(rng.uniform(-50, 50, 37))
    force = rng.normal(0, 1, (37, 3)) * 10.0 ** rng.integers(-9, 9, (37, 3))
    force[3, 1] = 0.0
    force[4, 2] = -0.0
    p = tmp_path / "tf.txt"
    io.write_table(p, grid, force)
    assert p.read_text() == O.tf_table_text(grid, force)


@pytest.mark.parametrize("num_types", [1, 5])
def test_read_table_kat(tmp_path, num_types):
    io = _lib_io()
    grid, force = _kat(num_types)
    p = tmp_path / "tf.txt"
    p.write_text(O.tf_table_text(grid, force))
    g2, f2, bw = io.read_table(p)
    og, of, obw = O.tf_table_parse(p.read_text())
    assert f2.shape == (100, num_types)
    np.testing.assert_array_equal(g2, og)
    np.testing.assert_array_equal(f2, of)
    assert bw == obw
    _float_eq(f2, force)


def test_read_table_random_values_bit_exact_with_oracle(tmp_path):
    io = _lib_io()
    rng = np.random.default_rng(11)
    grid = np.sort(rng.uniform(0, 30, 200))
    force = rng.normal(0, 3, (200, 4))
    p = tmp_path / "tf.txt"
    p.write_text(O.tf_table_text(grid, force))
    g2, f2, bw = io.read_table(p)
    og, of, obw = O.tf_table_parse(p.read_text())
    np.testing.assert_array_equal(g2, og)
    np.testing.assert_array_equal(f2, of)
    assert bw == obw


@pytest.mark.parametrize("text,max_forces", [
    ("", 10),                      # no grid line
    ("0.5\n1\n", 10),              # one bin (MRMD_HOST_ASSERT_GREATER(binNum, 1))
    ("0.5 1.5\n1 2 3\n", 10),      # force line longer than the grid
    ("0.5 1.5\n1\n", 10),          # shorter
    ("0.5 1.5\n1 2\n\n", 10),      # blank line counts as a (ragged) force line
    ("0.5 1.5\n1 x\n", 10),        # not a number
    ("0.5 1.5\n1 2\n3 4\n5 6\n", 2),  # more lines than maxNumForces
])
def test_read_table_rejects(tmp_path, text, max_forces):
    from mrmd_gb300 import MrmdError
    io = _lib_io()
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(MrmdError):
        io.read_table(p, max_forces)
    with pytest.raises(ValueError):
        O.tf_table_parse(text, max_forces)


def test_read_table_missing_file(tmp_path):
    from mrmd_gb300 import MrmdError
    with pytest.raises(MrmdError):
        _lib_io().read_table(tmp_path / "absent.txt")


def test_read_table_at_max_num_forces(tmp_path):
    io = _lib_io()
    grid, force = _kat(10, 8)
    p = tmp_path / "tf.txt"
    p.write_text(O.tf_table_text(grid, force))
    _, f2, _ = io.read_table(p, 10)
    np.testing.assert_array_equal(f2, force)


# ------------------------------------------------------------ device table --

@pytest.mark.gpu
@pytest.mark.parametrize("num_types", [1, 5])
def test_dump_restore_device_kat(tmp_path, num_types):
    """ThermoForce.test.cpp on the device table: setForce, dumpThermoForce,
    restoreThermoForce, then grid and forces EXPECT_FLOAT_EQ."""
    import mrmd_gb300 as M
    io = _lib_io()
    sd = M.Subdomain([1, 2, 3], [4, 6, 8], 0.5)
    ones = np.ones(num_types)
    tf1 = M.ThermodynamicForce(ones, sd, 3.0 / 100, ones)
    grid, force = _kat(num_types)
    tf1.setForce(force)
    _float_eq(tf1.getGrid(), grid)
    p = tmp_path / "tf.txt"
    io.dumpThermoForce(p, tf1, 0 if num_types == 1 else None)
    assert p.read_text() == O.tf_table_text(tf1.getGrid(), force, 0 if num_types == 1 else None)
    tf2 = io.restoreThermoForce(p, sd, ones, ones)
    assert (tf2.num_bins, tf2.num_types) == (100, num_types)
    _float_eq(tf2.getGrid(), tf1.getGrid())
    _float_eq(tf2.getForce(), tf1.getForce())


@pytest.mark.gpu
def test_restore_matches_oracle_table_and_mu(tmp_path):
    """A restored table equals the oracle's parse bit for bit, and getMuLeft /
    getMuRight over it equal the oracle's over the same table."""
    import mrmd_gb300 as M
    io = _lib_io()
    rng = np.random.default_rng(3)
    grid = O.tf_grid(0.0, 24.0, 48)
    force = rng.normal(0, 2, (48, 2))
    p = tmp_path / "tf.txt"
    p.write_text(O.tf_table_text(grid, force))
    sd = M.Subdomain([0, 0, 0], [24, 8, 8], 1.0)
    tf = io.restoreThermoForce(p, sd, [0.8, 0.8], [1.0, 0.5], max_num_forces=2)
    _, of, bw = O.tf_table_parse(p.read_text())
    np.testing.assert_array_equal(tf.getForce(), of)
    osd = O.subdomain([0, 0, 0], [24, 8, 8], 1.0)
    otf = O.ThermodynamicForce([0.8, 0.8], osd, bw, [1.0, 0.5])
    otf.force[:] = of
    l1, r1 = tf.getMu()
    l2, r2 = otf.mu()
    np.testing.assert_array_equal(l1, l2)
    np.testing.assert_array_equal(r1, r2)


@pytest.mark.gpu
def test_restore_rejects_mismatched_extents(tmp_path):
    import mrmd_gb300 as M
    io = _lib_io()
    grid, force = _kat(2)
    p = tmp_path / "tf.txt"
    p.write_text(O.tf_table_text(grid, force))
    sd = M.Subdomain([1, 2, 3], [4, 6, 8], 0.5)
    with pytest.raises(M.MrmdError):       # two force lines, three types
        io.restoreThermoForce(p, sd, [1, 1, 1], [1, 1, 1])
    wide = M.Subdomain([1, 2, 3], [7, 6, 8], 0.5)
    with pytest.raises(M.MrmdError):       # 100 bins in the file, 200 in the subdomain
        io.restoreThermoForce(p, wide, [1, 1], [1, 1])
