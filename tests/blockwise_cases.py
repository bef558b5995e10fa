"""The reference's blockwise test setup (test/test_xblockwise_reducer.cpp:95-140):
an int array (21, 10, 5), iota from -5 with +10 on odd flat indices, blocks
(5, 4, 2), the axis sets below, with keep_dims and with the immediate
strategy (same values as lazy)."""
import numpy as np

SHAPE = (21, 10, 5)
BLOCK = (5, 4, 2)
AXES = [(0,), (1,), (2,), (0, 1), (0, 2), (0, 1, 2)]
OPS = ["sum", "prod", "amin", "amax", "mean", "variance", "stddev",
       "norm_l0", "norm_l1", "norm_l2", "norm_sq", "norm_linf"]
P_OPS = ["norm_lp_to_p", "norm_lp"]


def input_exp() -> np.ndarray:
    x = np.arange(-5, -5 + int(np.prod(SHAPE)), dtype=np.int32)
    x[1::2] += 10
    return x.reshape(SHAPE)
