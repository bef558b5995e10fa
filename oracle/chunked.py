"""Restatement of the reference's chunk grid and chunk-by-chunk assignment —
test infrastructure only (tests use it as the checker; the library never
does).

  * chunks per dimension: s / cs, plus one edge chunk when s % cs > 0
    (xchunked_array::resize, include/xtensor/chunk/xchunked_array.hpp:601-625);
    every chunk is a full chunk_shape buffer;
  * element i of a dimension lives in chunk i / cs at i - (i / cs) * cs
    (get_chunk_indexes_in_dimension, :640-646);
  * chunks are visited in the grid's row-major order (xchunk_iterator::
    operator++, include/xtensor/chunk/xchunked_assign.hpp:283-306); chunk
    (g0, .., gR-1) covers range(g * cs, min((g + 1) * cs, s)) of the array
    (fill_slice_vector, :362-372) and range(0, min(cs, s - g * cs)) of its
    buffer (get_chunk_slice_vector, :346-360);
  * assignment copies each chunk's region of the expression into the chunk's
    buffer (xchunked_semantic::assign_xexpression, :200-219); the rest of an
    edge chunk's buffer is not written.
"""
from __future__ import annotations

import itertools

import numpy as np


def grid_shape(shape, chunk_shape):
    return tuple(s // c + (1 if s % c > 0 else 0) for s, c in zip(shape, chunk_shape))


def chunk_index(shape, chunk_shape, idx):
    """(chunk coordinates, coordinates inside the chunk) of element idx."""
    of = tuple(int(i) // c for i, c in zip(idx, chunk_shape))
    inn = tuple(int(i) - o * c for i, o, c in zip(idx, of, chunk_shape))
    return of, inn


def chunk_regions(shape, chunk_shape):
    """[(grid coordinates, array slices, buffer slices)] in visiting order."""
    out = []
    for gc in itertools.product(*[range(g) for g in grid_shape(shape, chunk_shape)]):
        arr = tuple(slice(g * c, min((g + 1) * c, s)) for g, c, s in zip(gc, chunk_shape, shape))
        buf = tuple(slice(0, min(c, s - g * c)) for g, c, s in zip(gc, chunk_shape, shape))
        out.append((gc, arr, buf))
    return out


def assign_chunks(chunks, values: np.ndarray, chunk_shape):
    """Each chunk buffer (list in visiting order) receives its region of the
    dense `values`; returns the chunks."""
    for (gc, arr, buf), ch in zip(chunk_regions(values.shape, chunk_shape), chunks):
        ch[buf] = values[arr]
    return chunks


def to_dense(chunks, shape, chunk_shape, dtype) -> np.ndarray:
    out = np.empty(shape, dtype=dtype)
    for (gc, arr, buf), ch in zip(chunk_regions(shape, chunk_shape), chunks):
        out[arr] = ch[buf]
    return out
