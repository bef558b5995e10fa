"""Known answers of the reference's accumulator tests
(test/test_xaccumulator.cpp), shared by the oracle test and the GPU test.
Each entry: (name, input array, op, axis, expected array, expected dtype)."""
from __future__ import annotations

import numpy as np

# TEST(xaccumulator, four_d) input: arange(36) as (2, 3, 2, 3) doubles
_X4 = np.arange(36, dtype=np.float64).reshape(2, 3, 2, 3)
_LONG = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8], [9, 10, 11]], np.int64)

KATS = [
    # one_d (:22-33): short input, int result
    ("one_d", np.array([1, 2, 3, 4], np.int16), "cumsum", None, np.array([1, 3, 6, 10]), np.int32),
    ("one_d_axis", np.array([1, 2, 3, 4], np.int16), "cumsum", 0, np.array([1, 3, 6, 10]), np.int32),
    # dim_one (:35-44)
    ("dim_one", np.array([[5.0, 6.0, 7.0]]), "cumsum", 0, np.array([[5.0, 6.0, 7.0]]), np.float64),
    ("dim_one_t", np.array([[5.0], [6.0], [7.0]]), "cumsum", 1, np.array([[5.0], [6.0], [7.0]]), np.float64),
    # four_d (:46-145): flattened row-major, and every axis
    ("four_d_flat", _X4, "cumsum", None, np.cumsum(np.arange(36.0)), np.float64),
    ("four_d_0", _X4, "cumsum", 0,
     np.array([[[[0, 1, 2], [3, 4, 5]], [[6, 7, 8], [9, 10, 11]], [[12, 13, 14], [15, 16, 17]]],
               [[[18, 20, 22], [24, 26, 28]], [[30, 32, 34], [36, 38, 40]], [[42, 44, 46], [48, 50, 52]]]],
              np.float64), np.float64),
    ("four_d_1", _X4, "cumsum", 1,
     np.array([[[[0, 1, 2], [3, 4, 5]], [[6, 8, 10], [12, 14, 16]], [[18, 21, 24], [27, 30, 33]]],
               [[[18, 19, 20], [21, 22, 23]], [[42, 44, 46], [48, 50, 52]], [[72, 75, 78], [81, 84, 87]]]],
              np.float64), np.float64),
    ("four_d_2", _X4, "cumsum", 2,
     np.array([[[[0, 1, 2], [3, 5, 7]], [[6, 7, 8], [15, 17, 19]], [[12, 13, 14], [27, 29, 31]]],
               [[[18, 19, 20], [39, 41, 43]], [[24, 25, 26], [51, 53, 55]], [[30, 31, 32], [63, 65, 67]]]],
              np.float64), np.float64),
    ("four_d_3", _X4, "cumsum", 3,
     np.array([[[[0, 1, 3], [3, 7, 12]], [[6, 13, 21], [9, 19, 30]], [[12, 25, 39], [15, 31, 48]]],
               [[[18, 37, 57], [21, 43, 66]], [[24, 49, 75], [27, 55, 84]], [[30, 61, 93], [33, 67, 102]]]],
              np.float64), np.float64),
    ("four_d_m1", _X4, "cumsum", -1,
     np.array([[[[0, 1, 3], [3, 7, 12]], [[6, 13, 21], [9, 19, 30]], [[12, 25, 39], [15, 31, 48]]],
               [[[18, 37, 57], [21, 43, 66]], [[24, 49, 75], [27, 55, 84]], [[30, 61, 93], [33, 67, 102]]]],
              np.float64), np.float64),
    # xtensor (:147-155)
    ("xtensor_2d", np.array([[1.0, 2, 3], [4, 5, 6]]), "cumsum", 0, np.array([[1.0, 2, 3], [5, 7, 9]]), np.float64),
    # cumprod (:164-178)
    ("cumprod_flat", _LONG, "cumprod", None, np.zeros(12, np.int64), np.int64),
    ("cumprod_0", _LONG, "cumprod", 0, np.array([[0, 1, 2], [0, 4, 10], [0, 28, 80], [0, 280, 880]]), np.int64),
    ("cumprod_1", _LONG, "cumprod", 1, np.array([[0, 0, 0], [3, 12, 60], [6, 42, 336], [9, 90, 990]]), np.int64),
    # empty_array (:196-210)
    ("empty_flat", np.ones((3, 4, 0)), "cumsum", None, np.zeros((0,)), np.float64),
    ("empty_2", np.ones((3, 4, 0)), "cumsum", 2, np.zeros((3, 4, 0)), np.float64),
    ("empty_1", np.ones((3, 4, 0)), "cumsum", 1, np.zeros((3, 4, 0)), np.float64),
]


def nan_equivalence_cases():
    """test/test_xnan_functions.cpp:152-172: nancumsum(a with NaNs) equals
    cumsum of the array with the NaNs replaced by 0 (nancumprod: by 1)."""
    g = np.random.default_rng(5)
    a = g.standard_normal((4, 5, 6))
    a[g.random(a.shape) < 0.2] = np.nan
    return a
