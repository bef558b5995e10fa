/*
 * xtg.h — C ABI of the GB300 evaluator for xtensor's assign + reduce hot path.
 *
 * Everything here is plain C: pointers, sizes, POD structs, status codes.
 * No C++ exceptions and no torch types cross this boundary.  A caller lowers
 * an xtensor expression tree (an `xfunction` over containers / strided views,
 * optionally wrapped by an `xreducer`) into an `xtg_expr` — a postfix list of
 * nodes plus up to XTG_MAX_LEAVES leaf arrays in device memory — and hands it
 * to xtg_assign / xtg_reduce / xtg_argreduce.  The library evaluates the whole
 * tree in one fused sm_103a kernel (compiled once per tree *shape* and cached),
 * with broadcasting folded into per-leaf stride arithmetic exactly as
 * xtensor's steppers do it.
 *
 * Reference interfaces replaced (paths inside xtensor 0.27.1):
 *   xtg_assign      <- xt::assign_xexpression / xexpression_assigner<Tag>::assign_data
 *                      include/xtensor/core/xassign.hpp:214-226, 439-478, 480-486
 *   xtg_broadcast_shape
 *                   <- xfunction::broadcast_shape / xt::broadcast_shape
 *                      include/xtensor/core/xfunction.hpp:709-727,
 *                      include/xtensor/core/xstrides.hpp:738-794
 *   xtg_reduce      <- xt::reduce + xreducer_stepper::aggregate(_impl) and
 *                      reduce_immediate; front-ends sum/prod/amax/amin/mean/
 *                      variance/stddev/norm_*
 *                      include/xtensor/reducers/xreducer.hpp:289-565, 987-1079, 1778-1868
 *                      include/xtensor/core/xmath.hpp:367-423, 777-811, 1803-1911, 2033-2180
 *                      include/xtensor/reducers/xnorm.hpp:397-526
 *   xtg_argreduce   <- xt::argmax / xt::argmin (arg_func_impl)
 *                      include/xtensor/misc/xsort.hpp:1158-1296
 *   xtg_assign_reduce
 *                   <- the pair `E = e; r = reduce(E, axes)` (assign_xexpression
 *                      then reduce), one pass where the plan allows
 *   xtg_accumulate  <- xt::cumsum / cumprod / nancumsum / nancumprod
 *                      (xt::accumulate, accumulator_impl)
 *                      include/xtensor/reducers/xaccumulator.hpp:154-367
 *                      include/xtensor/core/xmath.hpp:2248-2301, 2363-2391, 2592-2645
 *   xtg_npy_*       <- xt::load_npy / xt::dump_npy (include/xtensor/io/xnpy.hpp:
 *                      237-450, 674-800)
 *   xtg_blockwise_* <- xt::blockwise::* (include/xtensor/reducers/xblockwise_reducer.hpp:269-533)
 *   xtg_chunked_*   <- xt::xchunked_array / xt::as_chunked assignment, reading and reductions
 *                      include/xtensor/chunk/xchunked_array.hpp:56-686,
 *                      include/xtensor/chunk/xchunked_assign.hpp:185-272,
 *                      include/xtensor/chunk/xchunked_view.hpp:77-176
 *   xtg_gather / xtg_scatter, xtg_filter* , xtg_masked_assign
 *                   <- reading and assigning through xt::index_view / filter /
 *                      filtration / masked_view
 *                      include/xtensor/views/xindex_view.hpp:54-206, 786-850
 *                      include/xtensor/views/xmasked_view.hpp:63-240
 *   xtg_batch_*     <- no counterpart (new batching layer over the same path)
 *   xtg_server_*    <- no counterpart (new request server over the same path)
 *
 * Strides are in ELEMENTS (as xtensor's strides are), may be zero (broadcast)
 * or negative (reversed views).  Shapes follow xtensor's row-major convention.
 */
#ifndef XTG_H
#define XTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XTG_MAX_RANK 8
#define XTG_MAX_LEAVES 8
#define XTG_MAX_NODES 48
#define XTG_MAX_SCALARS 16

/* ---- status codes (xtensor throws; the ABI returns) ------------------------
 * XTG_ERR_BROADCAST  <- xt::broadcast_error        (core/xexception.hpp:122-135)
 * XTG_ERR_AXIS       <- std::runtime_error "Reducing axes should be sorted/…"
 *                       (reducers/xreducer.hpp:338-350, 1426-1440)
 * XTG_ERR_OUT_OF_RANGE <- std::out_of_range from normalize_axis
 *                       (core/xexception.hpp:287-297, utils/xutils.hpp:349-395)
 */
typedef enum {
    XTG_OK = 0,
    XTG_ERR_INVALID = 1,       /* malformed argument (null pointer, bad rank, bad dtype) */
    XTG_ERR_BROADCAST = 2,     /* incompatible shapes */
    XTG_ERR_AXIS = 3,          /* unsorted / duplicate / out-of-bounds reduction axes */
    XTG_ERR_OUT_OF_RANGE = 4,  /* axis outside [-rank, rank) */
    XTG_ERR_SHAPE = 5,         /* destination shape does not match the expression */
    XTG_ERR_CUDA = 6,          /* CUDA runtime / driver error */
    XTG_ERR_JIT = 7,           /* kernel compilation failed */
    XTG_ERR_OOM = 8,           /* device allocation failed or admission refused for memory */
    XTG_ERR_UNSUPPORTED = 9,   /* a combination this build does not lower */
    XTG_ERR_TIMEOUT = 10,      /* a bounded wait ran out */
    XTG_ERR_REJECTED = 11,     /* server admission rejected the request */
    XTG_ERR_CANCELLED = 12,    /* request cancelled before it ran */
    XTG_ERR_NOT_FOUND = 13     /* unknown request id / handle */
} xtg_status;

/* ---- element types ------------------------------------------------------- */
typedef enum {
    XTG_BOOL = 0,
    XTG_INT8 = 1,
    XTG_UINT8 = 2,
    XTG_INT16 = 3,
    XTG_UINT16 = 4,
    XTG_INT32 = 5,
    XTG_UINT32 = 6,
    XTG_INT64 = 7,
    XTG_UINT64 = 8,
    XTG_BFLOAT16 = 9,  /* storage type; arithmetic on it is carried out in float32 */
    XTG_FLOAT32 = 10,
    XTG_FLOAT64 = 11,
    XTG_NUM_DTYPES = 12
} xtg_dtype;

/* ---- expression node opcodes (postfix) -------------------------------------
 * Binary/unary opcodes mirror xtensor's functors (core/xoperation.hpp:104-143,
 * core/xmath.hpp:295-341, 589-602, 1101-1108).  A node's `dtype` is its
 * result type under C++ usual arithmetic conversions (what `decltype(f(a,b))`
 * gives for the functor in the reference); operands are converted to it
 * before the operation, comparisons/logical ops compute in the common type of
 * their operands and produce XTG_BOOL.
 */
typedef enum {
    XTG_OP_LEAF = 0,      /* arg = leaf index */
    XTG_OP_SCALAR = 1,    /* imm holds the value, dtype its type (xscalar) */
    /* unary */
    XTG_OP_NEG = 10, XTG_OP_POS, XTG_OP_EXP, XTG_OP_LOG, XTG_OP_SQRT, XTG_OP_ABS,
    XTG_OP_SQUARE, XTG_OP_SIN, XTG_OP_COS, XTG_OP_TANH, XTG_OP_LOGICAL_NOT,
    XTG_OP_BIT_NOT, XTG_OP_CAST,
    /* binary */
    XTG_OP_ADD = 40, XTG_OP_SUB, XTG_OP_MUL, XTG_OP_DIV, XTG_OP_MOD,
    XTG_OP_MAXIMUM, XTG_OP_MINIMUM,
    XTG_OP_LT, XTG_OP_LE, XTG_OP_GT, XTG_OP_GE, XTG_OP_EQ, XTG_OP_NE,
    XTG_OP_LOGICAL_AND, XTG_OP_LOGICAL_OR, XTG_OP_BIT_AND, XTG_OP_BIT_OR, XTG_OP_BIT_XOR,
    XTG_OP_POW,
    /* ternary: where(cond, a, b)  (conditional_ternary, core/xoperation.hpp:127-143) */
    XTG_OP_WHERE = 70,
    /* keep-dims row reductions over the last `arg` axes of the expression
     * shape, broadcast back over those axes.  They express
     * `x - mean(x, {trailing}, keep_dims)` style trees so that statistics and
     * the surrounding elementwise work run in one pass.  aux/imm.i = ddof for
     * RVAR / RSTD. */
    XTG_OP_RSUM = 80, XTG_OP_RMEAN, XTG_OP_RVAR, XTG_OP_RSTD, XTG_OP_RMAX, XTG_OP_RMIN
} xtg_opcode;

typedef union {
    double f;
    int64_t i;
    uint64_t u;
} xtg_value;

typedef struct {
    int32_t op;     /* xtg_opcode */
    int32_t dtype;  /* result xtg_dtype */
    int32_t arg;    /* leaf index (LEAF), target dtype (CAST), axis count (R*) */
    int32_t aux;    /* ddof for RVAR/RSTD */
    xtg_value imm;  /* SCALAR value (f for float types, i/u for integers) */
} xtg_node;

/* A strided array in device memory (host memory for the oracle).
 * data points at element (0,…,0). */
typedef struct {
    void* data;
    int32_t dtype;
    int32_t rank;
    int64_t shape[XTG_MAX_RANK];
    int64_t strides[XTG_MAX_RANK];
} xtg_array;

typedef struct {
    int32_t n_nodes;
    int32_t n_leaves;
    xtg_node nodes[XTG_MAX_NODES];
    xtg_array leaves[XTG_MAX_LEAVES];
} xtg_expr;

/* ---- reductions -------------------------------------------------------------
 * Result-type and initial-value rules follow XTENSOR_REDUCER_FUNCTION
 * (core/xmath.hpp:367-423), mean_division (core/xmath.hpp:1828-1835),
 * variance (core/xmath.hpp:2082-2103) and XTENSOR_NORM_FUNCTION
 * (reducers/xnorm.hpp:397-437). */
typedef enum {
    XTG_RED_SUM = 0, XTG_RED_PROD, XTG_RED_AMAX, XTG_RED_AMIN, XTG_RED_MEAN,
    XTG_RED_VARIANCE, XTG_RED_STDDEV, XTG_RED_NORM_L0, XTG_RED_NORM_L1,
    XTG_RED_NORM_SQ, XTG_RED_NORM_L2, XTG_RED_NORM_LINF,
    /* xtg_blockwise_reduce only (the blockwise norm_lp_to_p / norm_lp, which
     * take the exponent p): */
    XTG_RED_NORM_LP_TO_P, XTG_RED_NORM_LP
} xtg_reduce_op;

typedef enum {
    XTG_PREC_COMPENSATED = 0, /* float32/bf16: TwoSum double-float accumulation; float64: FP64 */
    XTG_PREC_PLAIN = 1        /* plain accumulation in the accumulator type */
} xtg_precision;

typedef struct {
    int32_t op;           /* xtg_reduce_op */
    int32_t n_axes;       /* -1: all axes (the no-axis overloads) */
    int64_t axes[XTG_MAX_RANK]; /* may be negative; normalized then checked sorted+unique */
    int32_t keep_dims;    /* xt::keep_dims */
    int32_t has_initial;  /* xt::initial(v) */
    xtg_value initial;    /* in the accumulator type's domain */
    int32_t acc_dtype;    /* -1 = default; else the `T` template argument (e.g. sum<int64_t>) */
    int32_t precision;    /* xtg_precision */
    int64_t ddof;         /* variance / stddev */
} xtg_reduce_desc;

typedef enum { XTG_ARGMAX = 0, XTG_ARGMIN = 1 } xtg_arg_op;

typedef void* xtg_stream; /* a cudaStream_t; NULL = legacy default stream */

enum { XTG_MEMCPY_H2D = 1, XTG_MEMCPY_D2H = 2, XTG_MEMCPY_D2D = 3, XTG_MEMCPY_DEFAULT = 4 };

/* ---- runtime --------------------------------------------------------------- */
const char* xtg_version(void);
const char* xtg_status_string(xtg_status s);
/* Message of the last failing call on this thread (empty if none). */
const char* xtg_last_error(void);
xtg_status xtg_init(int device);
xtg_status xtg_device_count(int* count);
xtg_status xtg_device_info(int* sm_count, int64_t* hbm_bytes, int* cc_major, int* cc_minor);
xtg_status xtg_mem_info(int64_t* free_bytes, int64_t* total_bytes);
xtg_status xtg_malloc(void** ptr, size_t bytes, xtg_stream stream); /* stream-ordered pool */
xtg_status xtg_free(void* ptr, xtg_stream stream);
xtg_status xtg_host_alloc(void** ptr, size_t bytes);                 /* pinned */
xtg_status xtg_host_free(void* ptr);
xtg_status xtg_memcpy(void* dst, const void* src, size_t bytes, int kind, xtg_stream stream);
xtg_status xtg_memset(void* dst, int value, size_t bytes, xtg_stream stream);
xtg_status xtg_stream_create(xtg_stream* stream);
xtg_status xtg_stream_destroy(xtg_stream stream);
xtg_status xtg_stream_sync(xtg_stream stream);
xtg_status xtg_device_sync(void);
size_t xtg_dtype_size(int32_t dtype);
/* Kernels never trap: a bounded wait that gives up, or an index-view
 * coordinate outside its array, sets a device error word and the kernel
 * skips the work.  This synchronises the device, reads and clears the word:
 * XTG_ERR_TIMEOUT (a wait gave up) or XTG_ERR_OUT_OF_RANGE (a coordinate). */
xtg_status xtg_check_device_errors(void);

/* CUDA events (timing on the launching stream). */
typedef void* xtg_event;
xtg_status xtg_event_create(xtg_event* ev);
xtg_status xtg_event_destroy(xtg_event ev);
xtg_status xtg_event_record(xtg_event ev, xtg_stream stream);
xtg_status xtg_event_sync(xtg_event ev);
xtg_status xtg_event_elapsed_ms(xtg_event start, xtg_event end, float* ms);
/* Work submitted to `stream` after this call waits until `ev` (as last
 * recorded) has completed: orders copies and evaluations across streams. */
xtg_status xtg_stream_wait_event(xtg_stream stream, xtg_event ev);

/* ---- shape algebra ----------------------------------------------------------- */
/* Broadcast shape of all leaves (right-aligned, size-1 / missing dims
 * broadcast), XTG_ERR_BROADCAST otherwise. */
xtg_status xtg_broadcast_shape(const xtg_expr* e, int32_t* rank, int64_t* shape);
/* Result dtype of the expression's root node after type checking. */
xtg_status xtg_expr_dtype(const xtg_expr* e, int32_t* dtype);
/* Output shape / dtype of a reduction (performs the axis checks). */
xtg_status xtg_reduce_shape(const xtg_expr* e, const xtg_reduce_desc* rd,
                            int32_t* rank, int64_t* shape, int32_t* out_dtype);
/* Accumulator dtype a reduction computes its sum in (the reference's
 * init-value/functor result type). */
xtg_status xtg_reduce_acc_dtype(const xtg_expr* e, const xtg_reduce_desc* rd, int32_t* acc_dtype);

/* ---- evaluation (the hot path) -------------------------------------------------
 * out must already have the broadcast shape (the container resize of
 * xassign.hpp:570-607 is the caller's), any strides.  A destination that
 * overlaps a leaf is only safe when it aliases it element-for-element (same
 * data pointer and strides), which is what computed assignment (`a += e`)
 * produces; the xt:: surface evaluates into a temporary otherwise. */
xtg_status xtg_assign(const xtg_expr* e, const xtg_array* out, xtg_stream stream);
xtg_status xtg_reduce(const xtg_expr* e, const xtg_reduce_desc* rd,
                      const xtg_array* out, xtg_stream stream);
/* has_axis = 0: index into the flattened (row-major) expression. */
xtg_status xtg_argreduce(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis,
                         const xtg_array* out, xtg_stream stream);
/* Assignment followed by a reduction of its result, in one pass where the
 * plan allows:  out_e = e  (as xtg_assign), then  out_r = reduce(rd, out_e)
 * (as xtg_reduce on out_e).  Replaces the pair of reference calls
 * `xt::xarray<T> E = e;` (assign_xexpression, core/xassign.hpp:214-226) and
 * `auto r = xt::sum(E, axes);` (reduce, reducers/xreducer.hpp:987-1079) at
 * one read of e's leaves and one write of E and r: when the reduction is a
 * row plan (reduced run contiguous), the tree has no row statistics and out_e
 * shares no memory with the leaves, one kernel stores every evaluated element
 * and folds it; otherwise the two evaluations run in order. */
xtg_status xtg_assign_reduce(const xtg_expr* e, const xtg_array* out_e, const xtg_reduce_desc* rd,
                             const xtg_array* out_r, xtg_stream stream);
/* The four reducers xt::sum, xt::mean, xt::variance (rd->ddof) and
 * xt::norm_l2 of one expression over rd's axes (rd->op is ignored; any
 * destination may be null) — core/xmath.hpp:367-423, 1828-1911, 2082-2103 and
 * reducers/xnorm.hpp:494-526 called one after the other on the same operand.
 * When the plan streams (a full reduction of one contiguous float32 / bf16
 * array in 16-byte vectors) the leaves are read once and each result equals
 * the corresponding xtg_reduce call bit for bit (its accumulator sees the
 * same values in the same order); otherwise the four reductions run in turn. */
xtg_status xtg_reduce_moments(const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* sum,
                              const xtg_array* mean, const xtg_array* variance, const xtg_array* norm_l2,
                              xtg_stream stream);

/* ---- accumulators ----------------------------------------------------------------------
 * Cumulative sum / product of an expression along `axis` (has_axis = 1; the
 * result has the expression's shape) or over its row-major flattening
 * (has_axis = 0; the result is 1-D of the expression's size).  The element
 * type is the accumulation type: acc_dtype (the reference's template
 * argument T, -1 = none) or the expression's value type, combined with the
 * value type as plus / multiplies would (short -> int, float -> float,
 * xt::cumsum<double>(float) -> double).  Elements fold sequentially in that
 * type; the nan variants start from NaN -> 0 / 1 and skip NaN operands.
 * An axis outside [-rank, rank) is XTG_ERR_AXIS ("Axis larger than
 * expression dimension in accumulator.").
 * Order of evaluation: along a non-innermost axis, and along the innermost
 * axis of expressions with many rows, each output element is folded in the
 * reference's sequential order (float results bit-identical); a few long
 * rows (and the flattened form) are cut into segments scanned from their
 * prefixes in a fixed order (reproducible run to run); float32 partial
 * results carry a double-float (TwoSum / TwoProd) error term, so they stay
 * within a few ulp of the exact prefix. */
typedef enum {
    XTG_ACC_CUMSUM = 0, XTG_ACC_CUMPROD = 1, XTG_ACC_NANCUMSUM = 2, XTG_ACC_NANCUMPROD = 3
} xtg_acc_op;
xtg_status xtg_accumulate_shape(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                                int32_t* rank, int64_t* shape, int32_t* dtype);
xtg_status xtg_accumulate(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                          const xtg_array* out, xtg_stream stream);

/* ---- .npy files ----------------------------------------------------------------------------
 * The NumPy format of the reference's load_npy / dump_npy: versions 1.0 and
 * 2.0, typestrings |b1 |i1 |u1 <i2 <u2 <i4 <u4 <i8 <u8 <f4 <f8 on a
 * little-endian host, C or Fortran order.  Data streams between the file (or
 * a host buffer) and device memory through pinned staging buffers, several
 * host threads each reading / writing its own chunks while the previous
 * chunk is in flight over the link.
 * Errors carry the reference's messages: XTG_ERR_INVALID for
 * "io error: failed to open a file.", "this file do not have a valid npy
 * format.", "unsupported file format version", "invalid header",
 * "missing 'descr' key", "invalid typestring", "invalid shape", "Cast error:
 * formats not matching <file> vs <requested>", "Cast error: layout mismatch
 * between npy file and requested layout."; XTG_ERR_SHAPE for a destination
 * whose shape differs from the file's; XTG_ERR_UNSUPPORTED for bfloat16
 * (no NumPy typestring) and rank > XTG_MAX_RANK. */
typedef struct {
    char descr[16];        /* the typestring as written, e.g. "<f8" */
    int32_t dtype;         /* the xtg_dtype written with that typestring here, -1 if none */
    int32_t fortran_order;
    int32_t version;       /* 1 or 2 */
    int32_t rank;
    int64_t shape[XTG_MAX_RANK];
    int64_t data_offset;   /* bytes of magic, version, length and header */
    int64_t data_bytes;    /* product of the shape times the item size */
} xtg_npy_header;
typedef enum { XTG_LAYOUT_DYNAMIC = 0, XTG_LAYOUT_ROW_MAJOR = 1, XTG_LAYOUT_COLUMN_MAJOR = 2 } xtg_layout;

xtg_status xtg_npy_info(const char* path, xtg_npy_header* h);
/* The header bytes dump_npy writes before the data (host only; *len gets
 * the size, nothing written when buf is NULL). */
xtg_status xtg_npy_format_header(int32_t dtype, int32_t fortran_order, int32_t rank, const int64_t* shape,
                                 char* buf, size_t cap, size_t* len);
xtg_status xtg_npy_info_buffer(const void* buf, size_t len, xtg_npy_header* h);
/* Reads the file into `out` (device memory, the file's shape, any strides).
 * The type check and the `layout` check are load_npy<T, L>'s, T being
 * out->dtype. */
xtg_status xtg_npy_load(const char* path, const xtg_array* out, int32_t layout, xtg_stream stream);
xtg_status xtg_npy_load_buffer(const void* buf, size_t len, const xtg_array* out, int32_t layout, xtg_stream stream);
/* Writes `in` with dump_npy's header and padding: a C-order file of its
 * dtype and shape, or a Fortran-order one when `in` is column-major
 * contiguous with rank > 1 and not also row-major contiguous; any other
 * strided `in` is evaluated into a row-major copy first.  Both return after
 * the bytes are in the file / buffer. */
xtg_status xtg_npy_save(const char* path, const xtg_array* in, xtg_stream stream);
/* *len receives the size of the whole file image; nothing is written when
 * buf is NULL; cap < *len is XTG_ERR_INVALID. */
xtg_status xtg_npy_save_buffer(const xtg_array* in, void* buf, size_t cap, size_t* len, xtg_stream stream);

/* ---- blockwise reducers ---------------------------------------------------------------------
 * xt::blockwise::sum / prod / amin / amax / mean / variance / stddev / norm_l0 /
 * norm_l1 / norm_l2 / norm_sq / norm_linf / norm_lp_to_p / norm_lp
 * (reducers/xblockwise_reducer.hpp:269-533, xblockwise_reducer_functors.hpp):
 * per-block results merged in block order (+=, *=, minimum / maximum, the
 * pairwise mean / variance update), then finalized (mean / factor, sqrt,
 * pow(., 1/p)).  `in` may be in device memory, or in host memory (pinned or
 * pageable, any dense strides) and larger than HBM: it streams through two
 * device buffers in slabs of whole blocks along its outermost dimension, the
 * copy of slab k+1 overlapping the reduction of slab k.  `out` (device) has
 * xtg_reduce_shape's shape and type; `p` is read by the lp ops only.
 * Unsupported: xt::initial and ddof (the reference's blockwise functors
 * take neither).  Returns once the host input is no longer read. */
xtg_status xtg_blockwise_reduce(const xtg_array* in, const int64_t* block_shape, const xtg_reduce_desc* rd, double p,
                                const xtg_array* out, xtg_stream stream);
/* Shape and type of that result. */
xtg_status xtg_blockwise_shape(const xtg_array* in, const xtg_reduce_desc* rd, int32_t* rank, int64_t* shape,
                               int32_t* out_dtype);

/* ---- chunked arrays ------------------------------------------------------------------------
 * A chunked array (xt::xchunked_array<xarray<xarray<T>>>, chunk/xchunked_array.hpp:56-686) in
 * device memory: `shape` cut into a grid of ceil(shape / chunk_shape) chunks, each a separate
 * row-major buffer of chunk_shape elements (the last chunk along a dimension ends inside its
 * buffer; the rest is padding, as the reference's resize makes it, :601-625).  `chunks` is a
 * host array of one device pointer per chunk, in the grid's row-major order.  Element
 * (i0, .., iR-1) is element (i % chunk_shape) of chunk (i / chunk_shape) (:640-646). */
typedef struct {
    void* const* chunks;
    int32_t dtype;
    int32_t rank;
    int64_t shape[XTG_MAX_RANK];
    int64_t chunk_shape[XTG_MAX_RANK];
} xtg_chunked;
/* dst = e, chunk by chunk (xchunked_semantic::assign_xexpression and computed_assign,
 * chunk/xchunked_assign.hpp:200-234; `a = e`, `noalias(a) = e`, `a += e`, `a += 2.` lower to it
 * with `a` itself a leaf).  Leaf i of e is chunked when chunked_leaves != NULL and
 * chunked_leaves[i] != NULL: its entry in e then only gives dtype and shape, and it must have
 * dst's shape and chunk shape.  Other leaves are dense device arrays broadcast to dst's shape.
 * One kernel for the whole grid; the padding of edge chunks is left untouched. */
xtg_status xtg_chunked_assign(const xtg_expr* e, const xtg_chunked* const* chunked_leaves, const xtg_chunked* dst,
                              xtg_stream stream);
/* dst (a dense device array of src's shape, any strides) = src: reading a chunked array
 * (`xt::xarray<T> b = a`, `noalias(b) = a`, `as_chunked(b, chunk_shape) = a`,
 * chunk/xchunked_view.hpp:77-176). */
xtg_status xtg_chunked_to_dense(const xtg_chunked* src, const xtg_array* dst, xtg_stream stream);
/* out = reduce(rd, src): the reducers of xtg_reduce (xt::sum / prod / amin / amax / mean /
 * variance / stddev / norm_*, reducers/xreducer.hpp:987-1079) over a chunked array, as the
 * blockwise reducers run them: each chunk's valid region reduced on the device, the results
 * of the chunks that share an output block folded in the grid's row-major order with the
 * blockwise merge (sum +=, prod *=, amin / amax, variance by the pairwise update), then
 * finalized.  out is a dense device array of the reduction's shape and result type.  Integer
 * results equal xtg_reduce's on the same values; floating-point sums associate by chunk.
 * xt::initial and ddof are rejected (XTG_ERR_UNSUPPORTED). */
xtg_status xtg_chunked_reduce(const xtg_chunked* src, const xtg_reduce_desc* rd, const xtg_array* out,
                              xtg_stream stream);

/* ---- index, filter and masked views ----------------------------------------------------
 * Assignment operators for writes through a view: dst = op(dst, value). */
typedef enum {
    XTG_SET = 0, XTG_SET_ADD = 1, XTG_SET_SUB = 2, XTG_SET_MUL = 3, XTG_SET_DIV = 4
} xtg_set_op;
/* out[k] = e[indices[k]] — reading an xt::index_view(e, indices).  indices:
 * device int64, n rows of rank(e) coordinates; out 1-D of n elements.
 * Coordinates outside e's shape are not read: the element is left as is and
 * the device error word is set (xtg_check_device_errors). */
xtg_status xtg_gather(const xtg_expr* e, const int64_t* indices, int64_t n, const xtg_array* out,
                      xtg_stream stream);
/* dst[indices[k]] = op(dst[indices[k]], src[k]) — assigning through an
 * index_view.  src is 1-D of n elements or broadcast to it (a scalar).
 * Repeated coordinates: each write happens, their order is unspecified. */
xtg_status xtg_scatter(const xtg_expr* src, const int64_t* indices, int64_t n, int32_t op, const xtg_array* dst,
                       xtg_stream stream);
/* Number of true elements of cond (synchronises the stream). */
xtg_status xtg_filter_count(const xtg_expr* cond, int64_t* count, xtg_stream stream);
/* out[k] = e[i_k], i_k the k-th position (row-major) where cond is true —
 * xt::filter(e, cond).  cond is broadcast to e's shape; out 1-D of
 * xtg_filter_count(cond) elements. */
xtg_status xtg_filter(const xtg_expr* e, const xtg_expr* cond, const xtg_array* out, xtg_stream stream);
/* dst[i_k] = op(dst[i_k], src[k]) — assigning through filter(dst, cond)
 * (src 1-D of the selected count) or through filtration(dst, cond) (src a
 * scalar). */
xtg_status xtg_filter_assign(const xtg_expr* src, const xtg_expr* cond, int32_t op, const xtg_array* dst,
                             xtg_stream stream);
/* dst[i] = mask[i] ? op(dst[i], src[i]) : dst[i] — assigning through
 * xt::masked_view(dst, mask); src and mask broadcast to dst's shape. */
xtg_status xtg_masked_assign(const xtg_expr* src, const xtg_expr* mask, int32_t op, const xtg_array* dst,
                             xtg_stream stream);

/* ---- batching ------------------------------------------------------------------------
 * No counterpart in the reference (a new layer over the same path).  Many
 * instances of ONE expression shape — same opcodes, leaf dtypes and ranks;
 * any sizes, strides and pointers — evaluated by one persistent launch whose
 * CTAs pull equal-work tiles (runs of rows of one instance) from a device
 * counter.  Each instance is a 2-D (rows, cols) evaluation (rank-1 leaves are
 * one row).  `rd` NULL: elementwise assignment into each instance's output;
 * otherwise a reduction over the last axis (rd->axes = {-1} or {rank-1}),
 * output (rows,) — e.g. sum(A * v + C, {1}) for 4096 uneven instances.
 * The template's leaves fix dtypes and ranks; xtg_batch_add binds each
 * instance's leaves in the template's leaf order.  xtg_batch_build uploads the
 * work list and picks the launch configuration (sub-warp group width, tile
 * size, CTAs per SM) — autotune = 1 measures the candidates on the instances
 * and caches the winner on disk per shape class; xtg_batch_capture records
 * one run into a CUDA graph that xtg_batch_replay launches. */
typedef struct xtg_batch xtg_batch;
typedef struct {
    int64_t instances;
    int64_t tiles;
    int64_t elements;
    int64_t algorithmic_bytes; /* leaves read once + outputs written once */
    int32_t group_lanes;
    int32_t unroll;
    int32_t ctas_per_sm;
    int32_t tuned;             /* 0 default, 1 measured now, 2 from the on-disk cache */
    int64_t tile_elems;
    int32_t graph_ready;
    int32_t pad;
} xtg_batch_info;
xtg_status xtg_batch_create(const xtg_expr* templ, const xtg_reduce_desc* rd, xtg_batch** b);
xtg_status xtg_batch_add(xtg_batch* b, const xtg_array* leaves, int32_t n_leaves, const xtg_array* out);
xtg_status xtg_batch_build(xtg_batch* b, int32_t autotune, xtg_stream stream);
xtg_status xtg_batch_run(xtg_batch* b, xtg_stream stream);
xtg_status xtg_batch_capture(xtg_batch* b, xtg_stream stream); /* stream must not be NULL */
xtg_status xtg_batch_replay(xtg_batch* b, xtg_stream stream);
xtg_status xtg_batch_get_info(const xtg_batch* b, xtg_batch_info* info);
xtg_status xtg_batch_destroy(xtg_batch* b);

/* ---- request server -------------------------------------------------------------------
 * No counterpart in the reference.  A request is one evaluation on operands
 * already resident in device memory: an assignment (out = expr), a reduction
 * (out = reduce(expr, rd)) or an arg-reduction.  xtg_server_submit never
 * blocks on the GPU: a scheduler thread admits pending requests while the
 * in-flight limit and the HBM budget allow (a request's cost is its declared
 * workspace plus the scratch its plan needs), groups admitted small requests
 * of the same tree shape into one batched launch, dispatches the others on a
 * pool of streams so their work overlaps, and completes requests from
 * stream callbacks.  Requests that arrive while others run join the next
 * admission round (continuous batching).  Latency = completion - submit. */
typedef struct xtg_server xtg_server;
typedef struct {
    int32_t streams;             /* concurrent CUDA streams (default 8) */
    int32_t max_inflight;        /* admitted, unfinished requests (default 256) */
    int64_t hbm_budget_bytes;    /* admission budget; 0: 90% of free HBM at creation */
    int64_t batch_max_elems;     /* requests up to this many elements may be grouped (default 1<<20) */
    int32_t batch_min_group;     /* smallest group launched as one batch (default 4) */
    int32_t pad;
} xtg_server_config;
enum { XTG_REQ_ASSIGN = 0, XTG_REQ_REDUCE = 1, XTG_REQ_ARGREDUCE = 2 };
typedef struct {
    int32_t kind;                /* XTG_REQ_* */
    int32_t arg_op;              /* argreduce: XTG_ARGMAX / XTG_ARGMIN */
    int32_t has_axis;
    int32_t pad;
    int64_t axis;
    int64_t workspace_bytes;     /* extra device memory the caller attributes to it */
    xtg_expr expr;
    xtg_reduce_desc rd;
    xtg_array out;
} xtg_request;
typedef struct {
    int32_t status;              /* xtg_status of the evaluation */
    int32_t batched;             /* 1 if it ran inside a grouped launch */
    double queue_ms;             /* submit -> dispatch */
    double total_ms;             /* submit -> completion */
} xtg_request_result;
typedef struct {
    int64_t submitted, completed, failed, rejected, cancelled, inflight, pending;
    int64_t waves, batched_requests, batch_launches;
    int64_t hbm_budget, hbm_reserved;
    double p50_ms, p99_ms, mean_ms;   /* over completed requests since the last reset */
    double dispatch_ms;               /* host time the dispatch threads spent launching work since the last reset */
} xtg_server_stats;
xtg_status xtg_server_create(const xtg_server_config* cfg, xtg_server** s);
xtg_status xtg_server_submit(xtg_server* s, const xtg_request* r, uint64_t* id);
/* timeout_ms < 0: wait forever; XTG_ERR_TIMEOUT when it runs out (the request
 * stays queued / in flight). */
xtg_status xtg_server_wait(xtg_server* s, uint64_t id, int64_t timeout_ms, xtg_request_result* res);
/* Cancels a request that has not been dispatched yet (XTG_ERR_NOT_FOUND otherwise). */
xtg_status xtg_server_cancel(xtg_server* s, uint64_t id);
xtg_status xtg_server_drain(xtg_server* s, int64_t timeout_ms);
xtg_status xtg_server_get_stats(xtg_server* s, xtg_server_stats* st);
xtg_status xtg_server_reset_stats(xtg_server* s);
xtg_status xtg_server_destroy(xtg_server* s);

/* Seeded synthetic data on the device (the benchmarks' inputs): element i of
 * a contiguous array gets a value from a counter-based generator keyed by
 * (seed, i), independent of the launch configuration.  dist: 0 uniform
 * [p0, p1), 1 normal(mean p0, sd p1), 2 sign-random lognormal(mu p0, sigma
 * p1), 3 integer uniform [p0, p1]. */
xtg_status xtg_fill_random(const xtg_array* a, int32_t dist, double p0, double p1, uint64_t seed, xtg_stream stream);

/* ---- reduction without allocation ------------------------------------------------
 * No counterpart in the reference.  For callers that must not allocate device
 * memory while they reduce: code whose device memory is owned by its own
 * allocator or budget (a framework that reserved the device's memory up
 * front, where an allocation by this library would fail or fragment it), and
 * loops with latency limits that must never enter an allocator.
 * Sum of the n contiguous float32 values at device pointer x, written to the
 * float at device pointer out — the same kernels and plan as xtg_reduce(sum,
 * all axes) on that array, so the result is bit-identical to it, with the
 * split-reduction partials in a static device array of
 * XTG_NOALLOC_SCRATCH_BYTES (every GPU the library is used on keeps it until
 * exit).  Inputs whose plan would need more partials than the array holds,
 * or more than 2^32 vectors, are rejected with XTG_ERR_UNSUPPORTED before any
 * launch.  The first call in a CUDA context resolves the array's address
 * there (cudaGetSymbolAddress, which also loads the library's device code).
 * A device reset or another context on the same device gets its own address.  All calls share the
 * array: calls whose kernels may overlap on the GPU (unordered streams) race
 * and must be serialised by the caller. */
#define XTG_NOALLOC_SCRATCH_BYTES (256u * 1024u)
xtg_status xtg_sum_f32_noalloc(const float* x, int64_t n, float* out, xtg_stream stream);

/* ---- kernel cache / tuning ------------------------------------------------------ */
typedef struct {
    int64_t compiles;       /* NVRTC compilations this process */
    int64_t disk_hits;      /* cubins loaded from the on-disk cache */
    int64_t memory_hits;    /* kernels found in the in-process cache */
    double compile_seconds; /* total time spent in NVRTC */
    int64_t launches;       /* kernels launched through this library */
} xtg_jit_stats;
xtg_status xtg_get_jit_stats(xtg_jit_stats* st);
/* Kernel names ("k_assign<...>;k_reduce_combine<...>") launched by the last
 * evaluation call on this thread — introspection for tests and tuning. */
const char* xtg_last_kernels(void);
/* Integer knobs: "assign.block", "assign.unroll", "assign.ctas_per_sm",
 * "reduce.block", "reduce.chunk", "transpose.tile", "batch.*" … ; value < 0 resets. */
xtg_status xtg_set_option(const char* key, int64_t value);
xtg_status xtg_get_option(const char* key, int64_t* value);

#ifdef __cplusplus
}
#endif
#endif /* XTG_H */
