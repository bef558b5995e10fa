"""The oracle's view semantics pinned to the reference's view tests
(test/test_xindex_view.cpp, test/test_xmasked_view.cpp) — CPU only."""
from __future__ import annotations

import numpy as np

from xtensor_gb300.device import HostArray as H
from oracle import oracle as O


def test_index_view_reads_and_writes():
    # TEST(xindex_view, indices) (:24-57) with a fixed e instead of rand
    e = np.arange(9, dtype=np.float64).reshape(3, 3) / 7.0
    idx = [[1, 1], [1, 2], [2, 2]]
    np.testing.assert_array_equal(O.index_view(H(e), idx), [e[1, 1], e[1, 2], e[2, 2]])
    d = e.copy()
    O.index_assign(d, idx, 3.0, "+=")
    assert d[1, 1] == e[1, 1] + 3
    O.index_assign(d, idx, 123.0, "=")
    assert d[1, 1] == d[1, 2] == d[2, 2] == 123
    O.index_assign(d, idx, H(np.array([3.0, 3.0, 3.0])), "=")
    assert d[2, 2] == 3


def test_filter_and_filtration():
    # TEST(xindex_view, boolean / fill / assign_scalar / filtration / filter)
    e = np.eye(3)
    assert O.filter(H(e), H(e) > 0)[0] == 1
    d = e.copy()
    O.filter_assign(d, H(e) > 0, 2.0, "+=")
    assert d[1, 1] == 3
    O.filter_assign(d, H(e) > 0, H(np.array([1.0, 2.0, 3.0])), "+=")
    assert d[1, 1] == 5 and d[2, 2] == 6
    f = np.eye(3)
    O.filter_assign(f, H(f) < 1, 2.0, "=")
    np.testing.assert_array_equal(f, [[1, 2, 2], [2, 1, 2], [2, 2, 1]])
    a = np.array([[1.0, 5, 3], [4, 5, 6]])
    O.filter_assign(a, H(a) >= 5, 2.0, "+=")
    np.testing.assert_array_equal(a, [[1, 7, 3], [4, 7, 8]])
    a = np.array([[1.0, 5, 3], [4, 5, 6]])
    b = np.array([[1.0, 5, 3], [4, 5, 6]])
    O.filter_assign(a, H(a) > 3, H(O.filter(H(b), H(b) > 3)), "+=")
    np.testing.assert_array_equal(a, [[1, 10, 3], [8, 10, 12]])
    # filter_column_major (:167-179), row-major half
    x = np.array([[[1, 3], [2, 4]], [[5, 7], [6, 8]]], np.int32)
    c = np.array([[[True, True], [False, False]], [[True, True], [False, False]]])
    np.testing.assert_array_equal(O.filter(H(x), H(c)), [1, 3, 5, 7])


def test_masked_view_assign():
    # TEST(xmasked_view, non_optional_data) (:189-213) and assign (:230-241)
    data = np.array([[1.0, -2, 3], [4, 5, -6], [7, 8, -9]])
    mask = np.array([[True, True, True], [True, False, False], [True, False, True]])
    O.masked_assign(data, H(mask), 3.65, "=")
    np.testing.assert_array_equal(data, [[3.65, 3.65, 3.65], [3.65, 5, -6], [3.65, 8, 3.65]])
    O.masked_assign(data, H(mask), 3.0, "+=")
    np.testing.assert_array_equal(data, [[6.65, 6.65, 6.65], [6.65, 5, -6], [6.65, 8, 6.65]])
    data = np.array([[1.0, -2, 3], [4, 5, -6], [7, 8, -9]])
    data2 = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6], [0.7, 0.8, 0.9]])
    O.masked_assign(data, H(mask), H(data2), "=")
    np.testing.assert_array_equal(data, [[0.1, 0.2, 0.3], [0.4, 5, -6], [0.7, 8, 0.9]])
    # TEST(xmasked_view, view) (:243-256): a masked row view
    d = np.array([[0, 1], [2, 3], [4, 5]], np.uint64)
    row = d[0]
    O.masked_assign(row, H(np.array([False, True])), 10, "+=")
    assert d[0, 0] == 0 and d[0, 1] == 11
