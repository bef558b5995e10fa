// xtg_params.h — kernel parameter blocks shared by the host planner and the
// device code (plain POD, no CUDA qualifiers, so g++ and NVRTC both see the
// same layout).  Shapes and strides are in elements; offsets are 64-bit.
#pragma once
#ifndef XTG_PARAMS_H
#define XTG_PARAMS_H

namespace xtg {

typedef long long i64;
typedef unsigned long long u64;
typedef unsigned int u32;

// Divisor for the multiply-and-shift division of the device code.
struct FastDiv {
    u32 d, m, l;
};

#define XTG_KMAX_RANK 8
#define XTG_KMAX_LEAVES 8
#define XTG_KMAX_SCAL 16

struct Scalars {
    u64 v[XTG_KMAX_SCAL];
};
// Iteration space: rank R dims; dim R-1 is the vectorised one.  `shape` holds
// extents with the innermost one in vectors; `fd` the matching divisors.
struct Space {
    i64 shape[XTG_KMAX_RANK];
    FastDiv fd[XTG_KMAX_RANK];
    i64 nvec;  // product of shape[] (innermost counted in vectors)
};

struct AssignParams {
    Space sp;
    void* out;
    i64 out_strides[XTG_KMAX_RANK];
    const void* leaf[XTG_KMAX_LEAVES];
    i64 leaf_strides[XTG_KMAX_LEAVES][XTG_KMAX_RANK];
    Scalars scal;
};

// Chunked evaluation (K12): the iteration space is one chunk (all chunks
// share its shape), repeated for every chunk of the grid; per chunk a table
// entry gives the leaves' and the destination's base pointers and the
// chunk's valid extents (edge chunks end inside their buffer).
struct ChunkEntry {
    const void* leaf[XTG_KMAX_LEAVES];
    void* out;
    i64 ext[XTG_KMAX_RANK];
};
// Chunks whose valid extents agree form a class (full chunks, the edge chunk
// along some dims, ...); a class's chunks occupy entries [first, first +
// count) of the table.  With PAD the launch has one class of padded chunks
// and the entries' extents bound the elements.
#define XTG_KCHUNK_CLS 8
struct ChunkClass {
    Space sp;          // one chunk of the class, innermost dim in vectors
    FastDiv fdn;       // divisor sp.nvec (32-bit launches)
    i64 first, count;
};
struct ChunkParams {
    ChunkClass cls[XTG_KCHUNK_CLS];
    int n_cls;
    const ChunkEntry* tab;
    i64 leaf_strides[XTG_KMAX_LEAVES][XTG_KMAX_RANK];  // within a chunk
    i64 out_strides[XTG_KMAX_RANK];
    Scalars scal;
};

struct TransposeParams {
    i64 sa, sb;            // extents of A and B
    i64 ntile_a, ntile_b;
    i64 n_tiles;           // nbatch * ntile_a * ntile_b
    i64 bshape[XTG_KMAX_RANK];  // batch dims (all except A and B), outer first
    int nbd;
    void* out;
    i64 oa, ob;            // destination strides along A, B
    i64 obs[XTG_KMAX_RANK];     // destination strides over batch dims
    const void* leaf[XTG_KMAX_LEAVES];
    i64 la[XTG_KMAX_LEAVES], lb[XTG_KMAX_LEAVES];
    i64 lbs[XTG_KMAX_LEAVES][XTG_KMAX_RANK];
    Scalars scal;
};

struct RedParams {
    i64 oshape[XTG_KMAX_RANK];
    FastDiv ofd[XTG_KMAX_RANK];
    i64 rshape[XTG_KMAX_RANK];
    FastDiv rfd[XTG_KMAX_RANK];
    i64 n_out;      // outputs (elements)
    i64 n_outv;     // output vectors (COL) or outputs (ROW)
    i64 n_red;      // reduced elements per output
    i64 n_redv;     // reduced vectors (ROW) or elements (COL)
    i64 chunk;      // reduced vectors/elements per split
    i64 nsplit;
    const void* leaf[XTG_KMAX_LEAVES];
    i64 lks[XTG_KMAX_LEAVES][XTG_KMAX_RANK];  // leaf strides over kept dims
    i64 lrs[XTG_KMAX_LEAVES][XTG_KMAX_RANK];  // leaf strides over reduced dims
    void* out;
    i64 ostr[XTG_KMAX_RANK];                  // output strides over kept dims
    void* partial;                            // nsplit > 1: n_out * nsplit states
    Scalars scal;
    double init_f;
    i64 init_i;
    int has_initial;
    double initial_f;
    i64 initial_i;
    double divisor;  // mean / variance divisor (already integer-divided like the reference)
    // fused assign + reduce (row kernel with ES != 0): every evaluated
    // element, converted to the destination type, is also stored at
    // eout + sum(kept index * eks) + sum(reduced index * ers)
    void* eout;
    i64 eks[XTG_KMAX_RANK];
    i64 ers[XTG_KMAX_RANK];
    int* err;  // streaming row kernel: set to 1 when a bounded wait gives up
    // one-pass moments (xtg_reduce_moments): mean, variance and norm_l2
    // destinations beside the sum's `out` (null: not wanted), and the
    // variance divisor (the mean's is `divisor`)
    void* out_more[3];
    double divisor2;
};

struct RowParams {
    i64 n_rows;
    i64 row_len;
    i64 oshape[XTG_KMAX_RANK];  // outer (row) dims
    const void* leaf[XTG_KMAX_LEAVES];
    i64 lo[XTG_KMAX_LEAVES][XTG_KMAX_RANK];  // leaf strides over outer dims
    i64 li[XTG_KMAX_LEAVES];                 // leaf stride along the row
    void* out;
    i64 oo[XTG_KMAX_RANK];
    i64 oi;
    Scalars scal;
    double div[XTG_KMAX_SCAL];  // per statistic divisor (mean: n, var: n - ddof)
    double rdiv[XTG_KMAX_SCAL]; // 1 / div (float64 rows multiply)
    double vfac[XTG_KMAX_SCAL]; // 1 / (row_len * div): float64 variance from n * sum of squared deviations
    int rdiv_e2[XTG_KMAX_SCAL]; // rdiv == 2^k: k + 100000, else 0 (float64 rows scale by the exponent)
    int vfac_e2[XTG_KMAX_SCAL]; // the same for vfac
    float fdiv[XTG_KMAX_SCAL];  // div as float (float32 rows divide in FP32)
    double rrow_len;            // 1 / row_len
    float frow_len;             // row_len as float
    // bulk-copy (TMA) variant: per-warp buffer layout in shared memory
    unsigned loff[XTG_KMAX_LEAVES];   // byte offset of each leaf's row inside a buffer
    unsigned lbytes[XTG_KMAX_LEAVES]; // bytes of one row of each leaf (multiple of 16)
    unsigned buf_bytes;               // bytes of one buffer (all leaves)
    int* err;                         // set to 1 when a bounded wait gives up
};

// Accumulators (cumsum / cumprod): the expression's iteration space as
// (outer, axis, inner), each part collapsed to one dimension.
struct ScanParams {
    i64 n_outer, len, n_inner;
    const void* leaf[XTG_KMAX_LEAVES];
    i64 lso[XTG_KMAX_LEAVES], lsa[XTG_KMAX_LEAVES], lsi[XTG_KMAX_LEAVES];  // leaf strides
    void* out;
    i64 oso, osa, osi;  // destination strides
    Scalars scal;
    i64 ntiles;         // segmented scan: tiles per row
    void* agg;          // segmented scan: one partial state (16 B) per segment
    i64 csum_off;       // segmented scan: byte offset from agg of the lanes' tile sums (0: none)
};

// Indexed evaluation through index_view / filter (gathers and scatters).
// MODE 0 gather (out[k] = e[idx row k]), 1 scatter (dst[idx row k] op= src[k]),
// 2 filter gather (out[P[i]-1] = e[i] where selected), 3 filter assign
// (dst[i] op= src[P[i]-1] where selected); P = inclusive count of the
// condition in row-major order.
struct IndexParams {
    i64 n;                                      // index rows (0, 1) or flat positions (2, 3)
    int rank;
    i64 shape[XTG_KMAX_RANK];                   // the indexed space (e: 0, 2; dst: 1, 3)
    FastDiv fd[XTG_KMAX_RANK];                  // row-major decode of flat positions (2, 3)
    const long long* idx;                       // n x rank coordinates (0, 1) or P (2, 3)
    const void* leaf[XTG_KMAX_LEAVES];
    i64 ls[XTG_KMAX_LEAVES][XTG_KMAX_RANK];     // value-tree leaf strides (0, 2: indexed space; 1, 3: dim 0)
    void* dst;
    i64 ds[XTG_KMAX_RANK];                      // out stride in ds[0] (0, 2) or dst strides (1, 3)
    Scalars scal;
    int* err;                                   // set when a coordinate is outside the shape
};

// Filters by tiles of 4096 row-major positions: the condition tree (c*) and
// the value tree (v*: the filtered expression, or the 1-D values assigned)
// with their own leaves and scalars.
struct FilterParams {
    i64 n;                                      // positions in the filtered shape
    i64 shape[XTG_KMAX_RANK];
    FastDiv fd[XTG_KMAX_RANK];
    const void* cleaf[XTG_KMAX_LEAVES];
    i64 cls[XTG_KMAX_LEAVES][XTG_KMAX_RANK];    // condition leaf strides over the shape
    const void* vleaf[XTG_KMAX_LEAVES];
    i64 vls[XTG_KMAX_LEAVES][XTG_KMAX_RANK];    // value leaves: over the shape (read) or dim 0 (assign)
    void* dst;
    i64 ds[XTG_KMAX_RANK];                      // out stride in ds[0] (read) or dst strides (assign)
    Scalars cscal, vscal;
    int* tcount;                                // selected per tile
    const long long* tincl;                     // inclusive selected count per tile
};

// Batched evaluation: many instances of one expression shape, each a 2-D
// (rows, cols) space with its own pointers and strides.
struct BatchInst {
    const void* leaf[XTG_KMAX_LEAVES];
    i64 rs[XTG_KMAX_LEAVES];  // leaf strides between rows (0: broadcast)
    i64 cs[XTG_KMAX_LEAVES];  // leaf strides between columns
    void* out;
    i64 ors, ocs;             // destination strides (reductions use ors only)
    i64 rows, cols;
    double divisor;           // mean divisor of a row
};
struct BatchTile {
    int inst;
    int nrows;
    i64 row0;
};
struct BatchParams {
    const BatchInst* inst;
    const BatchTile* tiles;
    i64 ntiles;
    int* counter;             // next tile; zeroed before every launch
    Scalars scal;
    double init_f;
    i64 init_i;
    int has_initial;
    double initial_f;
    i64 initial_i;
};
// Per-row finishing parameters (the fields the accumulators' finishers read).
struct FinP {
    double init_f;
    i64 init_i;
    int has_initial;
    double initial_f;
    i64 initial_i;
    double divisor;
    i64 n_red;
};

}  // namespace xtg
#endif
