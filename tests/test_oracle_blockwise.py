"""The blockwise restatement (oracle/blockwise.py) pinned to the reference's
own test: blockwise::<op>(x, block, axes, options) equals the plain reducer
<op>(x, axes, options) — exactly, except variance / stddev (allclose), as
test_xblockwise_reducer.cpp:95-215 checks."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import blockwise as B
from oracle import oracle as O
from xtensor_gb300.device import HostArray as H
from xtensor_gb300.expr import pow_, scalar

from blockwise_cases import AXES, BLOCK, OPS, P_OPS, input_exp


@pytest.mark.parametrize("keep_dims", [True, False])
@pytest.mark.parametrize("op", OPS)
def test_blockwise_equals_plain_reducer(op, keep_dims):
    x = input_exp()
    for axes in AXES:
        got = B.blockwise(op, x, BLOCK, list(axes), keep_dims)
        want = O.reduce(op, H(x), list(axes), keep_dims)
        assert got.dtype == want.dtype and got.shape == want.shape, (op, axes)
        if op in ("variance", "stddev"):
            np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-8)
        else:
            np.testing.assert_array_equal(got, want, err_msg=f"{op} {axes}")


@pytest.mark.parametrize("keep_dims", [True, False])
@pytest.mark.parametrize("op", P_OPS)
def test_blockwise_p_norms_equal_plain(op, keep_dims):
    """test_p_norm_values (:141-215) with p = 2: the plain norm_lp_to_p sums
    pow(abs(x), p) in double, norm_lp takes pow(., 1/p)."""
    x = input_exp()
    for axes in AXES:
        got = B.blockwise(op, x, BLOCK, list(axes), keep_dims, p=2.0)
        s = O.reduce("sum", pow_(H(np.abs(x)), scalar(2.0)), list(axes), keep_dims, acc_dtype="float64")
        want = s if op == "norm_lp_to_p" else np.power(s, 0.5)
        assert got.dtype == np.float64 and got.shape == want.shape
        np.testing.assert_allclose(got, want, rtol=1e-15)
