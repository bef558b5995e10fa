"""The chunk-grid restatement (oracle/chunked.py) pinned to the expectations of
the reference's own chunked-array tests (test/test_xchunked_array.cpp,
test/test_xchunked_view.cpp), on the CPU."""
from __future__ import annotations

import numpy as np

from oracle import chunked as OC


def test_grid_and_chunk_count():
    # test_xchunked_view.cpp:16-31 (iterate): shape {3, 4}, chunks {1, 2} -> 3 * 2 chunks
    assert OC.grid_shape((3, 4), (1, 2)) == (3, 2)
    assert len(OC.chunk_regions((3, 4), (1, 2))) == 6
    # edge chunks: {10, 10, 10} in {2, 3, 4} -> 5 x 4 x 3
    assert OC.grid_shape((10, 10, 10), (2, 3, 4)) == (5, 4, 3)
    # {2, 2, 2} in {2, 3, 4}: one chunk larger than the array (test_xchunked_array.cpp:50-53)
    assert OC.grid_shape((2, 2, 2), (2, 3, 4)) == (1, 1, 1)


def test_indexed_access_location():
    # test_xchunked_array.cpp:20-33: element {3, 9, 8} of {10, 10, 10} in {2, 3, 4}
    of, inn = OC.chunk_index((10, 10, 10), (2, 3, 4), (3, 9, 8))
    assert of == (1, 3, 2) and inn == (1, 0, 0)


def test_chunk_iterator_first_elements():
    # test_xchunked_array.cpp:138-168: chunk (i, j, k) of {10, 10, 10} in {2, 2, 2}
    # starts at a(2i, 2j, 2k), in row-major grid order; advancing twice from
    # the first chunk lands on the chunk starting at a(0, 0, 4)
    b = np.arange(1000, dtype=np.float64).reshape(10, 10, 10)
    chunks = OC.assign_chunks([np.zeros((2, 2, 2)) for _ in range(125)], b, (2, 2, 2))
    regions = OC.chunk_regions((10, 10, 10), (2, 2, 2))
    n = 0
    for i in range(5):
        for j in range(5):
            for k in range(5):
                assert regions[n][0] == (i, j, k)
                assert chunks[n][0, 0, 0] == b[2 * i, 2 * j, 2 * k]
                n += 1
    assert chunks[2][0, 0, 0] == b[0, 0, 4]


def test_assign_and_read_back():
    # test_xchunked_array.cpp:85-98: {{1..9}} in chunks {2, 2} iterates as 1..9
    a3 = np.arange(1.0, 10.0).reshape(3, 3)
    chunks = OC.assign_chunks([np.full((2, 2), -7.0) for _ in range(4)], a3, (2, 2))
    np.testing.assert_array_equal(OC.to_dense(chunks, (3, 3), (2, 2), np.float64), a3)
    # edge chunks keep their padding
    assert chunks[3][0, 0] == 9.0 and chunks[3][1, 1] == -7.0 and chunks[1][0, 1] == -7.0
    # test_xchunked_array.cpp:113-125: {3, 3} in {1, 2}; every chunk keeps the chunk shape
    c7 = OC.assign_chunks([np.zeros((1, 2)) for _ in range(6)], a3, (1, 2))
    assert all(c.shape == (1, 2) for c in c7)
    np.testing.assert_array_equal(OC.to_dense(c7, (3, 3), (1, 2), np.float64), a3)
