"""Interface numbering of the multidomain coupling (md_influence_matrix_param,
src/class_md/class_md.f90:1450-1680): the C ABI against the oracle.  No GPU."""
import numpy as np
import pytest

from oracle import md


@pytest.mark.parametrize("nd,periods,nint", [
    ((2, 2, 2), (0, 0, 0), ([15, 15], [15, 15], [15, 15])),
    ((3, 2, 1), (1, 0, 0), ([11, 13, 9], [15, 7], [9])),
    ((1, 1, 1), (1, 1, 0), ([9], [11], [13])),
    ((2, 3, 2), (0, 1, 1), ([47, 63], [63, 95, 47], [95, 63])),
])
def test_topology_matches_oracle(mf, nd, periods, nint):
    got = mf.md_topology(nd, periods, nint)
    ref = md.Topology(nd, periods, nint)
    assert got["it"] == ref.it
    assert got["ninf"] == ref.ninf
    assert np.array_equal(got["dm_int"], ref.dm_int)
    assert np.array_equal(got["kind"], ref.kind)
    assert np.array_equal(got["size"], ref.size)
    assert np.array_equal(got["offset"], ref.offset)


def test_topology_two_by_two_by_two_counts(mf):
    # 2x2x2 non periodic: 4 interfaces per direction, 12 in total
    got = mf.md_topology((2, 2, 2), (0, 0, 0), ([63, 63], [63, 63], [63, 63]))
    assert got["it"] == 12 and got["ninf"] == 12 * 63 * 63
