"""Restatement of the reference's blockwise reducers — test infrastructure only.

Follows include/xtensor/reducers/xblockwise_reducer.hpp:
  * init_shapes (:196-239): result shape / result chunk shape (kept axes
    take the block extent, reduced axes 1 or dropped);
  * assign_to / assign_to_chunk / compute_input_chunk_range (:129-194): for
    every result chunk, the input blocks of its reduced-axes range in
    row-major grid order, each reduced by `compute`, folded by `merge`, the
    chunk then `finalize`d;
and the functors of xblockwise_reducer_functors.hpp:25-500:
  * sum / prod: sum<value_type> / prod<value_type> per block, += / *=;
  * amin / amax: amin / amax per block, xt::minimum(block, result) /
    xt::maximum(block, result);
  * mean: sum<value_type> per block, +=, then /= static_cast<value_type>(factor);
  * variance / stddev: (variance<value_type>, mean<value_type>, weight) per
    block, the pairwise update in double, stddev takes the sqrt at the end;
  * norm_l0 / l1 / sq / l2 / linf: sum of not_equal(x, 0) / abs(x) /
    square(x), amax of abs(x); l2 takes the sqrt at the end;
  * norm_lp_to_p / norm_lp: sum<double>(pow(x, p)); lp takes pow(., 1/p).
Each block's reduction is the C oracle's plain reducer (oracle/xt_oracle.c),
so block results follow the reference's loop order; merges are numpy in the
functors' C++ types.
"""
from __future__ import annotations

import itertools

import numpy as np

from xtensor_gb300.device import HostArray as H
from xtensor_gb300.expr import abs_, not_equal, pow_, scalar, square

from . import oracle as O


def _trunc_div(a: np.ndarray, f: int, dt) -> np.ndarray:
    if np.dtype(dt).kind == "f":
        return (a / np.asarray(f, dtype=dt)).astype(dt)
    q = np.abs(a.astype(np.int64 if np.dtype(dt).kind == "i" else np.uint64)) // f
    return (np.sign(a) * q).astype(dt) if np.dtype(dt).kind == "i" else q.astype(dt)


def result_dtype(op, x, acc_dtype=None):
    if op in ("norm_lp_to_p", "norm_lp"):
        return np.dtype(np.float64)
    z = x.reshape(-1)[:1] if x.size else x
    return O.reduce(op, H(np.ascontiguousarray(z)), None, False, acc_dtype=acc_dtype).dtype


def blockwise(op: str, x: np.ndarray, block_shape, axes=None, keep_dims=False, p=2.0, acc_dtype=None):
    rank = x.ndim
    axes = list(range(rank)) if axes is None else sorted(a + rank if a < 0 else a for a in
                                                         ([axes] if isinstance(axes, int) else axes))
    R = result_dtype(op, x, acc_dtype)
    red = [d in axes for d in range(rank)]
    grid = [-(-x.shape[d] // block_shape[d]) if x.shape[d] else 0 for d in range(rank)]
    # result shape as the reducer's
    out_shape = [(1 if red[d] else x.shape[d]) for d in range(rank) if keep_dims or not red[d]]
    out = np.zeros(out_shape, dtype=R)
    kept = [d for d in range(rank) if not red[d]]

    def block_result(blk):
        hb = H(np.ascontiguousarray(blk))
        kw = dict(axes=axes, keep_dims=keep_dims)
        if op in ("sum", "prod", "mean"):
            return O.reduce("prod" if op == "prod" else "sum", hb, acc_dtype=R, **kw)
        if op in ("amin", "amax"):
            return O.reduce(op, hb, **kw)
        if op in ("variance", "stddev"):
            w = float(np.prod([blk.shape[a] for a in axes])) if axes else 1.0
            return (O.reduce("variance", hb, acc_dtype=R, **kw), O.reduce("mean", hb, acc_dtype=R, **kw), w)
        if op == "norm_l0":
            return O.reduce("sum", not_equal(hb, scalar(0, np.dtype(blk.dtype).name)), acc_dtype=R, **kw)
        if op == "norm_l1":
            return O.reduce("sum", abs_(hb), acc_dtype=R, **kw)
        if op in ("norm_sq", "norm_l2"):
            return O.reduce("sum", square(hb), acc_dtype=R, **kw)
        if op == "norm_linf":
            return O.reduce("amax", abs_(hb), acc_dtype=R, **kw)
        if op in ("norm_lp_to_p", "norm_lp"):
            return O.reduce("sum", pow_(hb, scalar(float(p))), acc_dtype=R, **kw)
        raise ValueError(op)

    kept_ranges = [range(grid[d]) for d in kept]
    red_ranges = [range(grid[d]) for d in axes]
    for kidx in itertools.product(*kept_ranges):
        first = True
        acc = mean_a = None
        n_a = 0.0
        for ridx in itertools.product(*red_ranges):
            sl = [slice(None)] * rank
            for d, i in zip(kept, kidx):
                sl[d] = slice(i * block_shape[d], (i + 1) * block_shape[d])
            for d, i in zip(axes, ridx):
                sl[d] = slice(i * block_shape[d], (i + 1) * block_shape[d])
            br = block_result(x[tuple(sl)])
            if op in ("variance", "stddev"):
                var_b, mean_b, n_b = br
                if first:
                    acc, mean_a, n_a = var_b.astype(R), mean_b.astype(R), n_b
                else:
                    va, ma = acc.astype(np.float64), mean_a.astype(np.float64)
                    vb, mb = var_b.astype(np.float64), mean_b.astype(np.float64)
                    new_mean = (n_a * ma + n_b * mb) / (n_a + n_b)
                    new_var = (n_a * va + n_b * vb + n_a * (ma - new_mean) * (ma - new_mean)
                               + n_b * (mb - new_mean) * (mb - new_mean)) / (n_a + n_b)
                    acc, mean_a = new_var.astype(R), new_mean.astype(R)
                    n_a += n_b
            elif first:
                acc = br.astype(R)
            elif op in ("amin",):
                acc = np.where(br < acc, br, acc).astype(R)
            elif op in ("amax", "norm_linf"):
                acc = np.where(br > acc, br, acc).astype(R)
            elif op == "prod":
                acc = (acc * br.astype(R)).astype(R)
            else:
                acc = (acc + br.astype(R)).astype(R)
            first = False
        if acc is None:
            continue
        # the result chunk
        osl = []
        for d in range(rank):
            if not red[d]:
                i = kidx[kept.index(d)]
                osl.append(slice(i * block_shape[d], (i + 1) * block_shape[d]))
            elif keep_dims:
                osl.append(slice(None))
        out[tuple(osl)] = acc
    # finalize (per chunk in the reference; elementwise, so once here)
    with np.errstate(all="ignore"):
        if op == "mean":
            factor = int(np.prod([x.shape[a] for a in axes])) if axes else 1
            out = _trunc_div(out, factor, R)
        elif op in ("stddev", "norm_l2"):
            out = np.sqrt(out).astype(R)
        elif op == "norm_lp":
            out = np.power(out, 1.0 / p).astype(R)
    return out
