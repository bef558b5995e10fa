/*
 * xt_baseline.c — compiled CPU port of the reference's code path for the
 * benchmark workloads.  TEST / BASELINE INFRASTRUCTURE ONLY: timed as the
 * CPU baseline by bench.py, which also checks the GPU results of its
 * benchmark steps against these routines' outputs; the routines themselves
 * are pinned to the oracle (xt_oracle.c) bit for bit on small seeded inputs
 * by tests/test_baseline_port.py.  The product library never uses it.
 *
 * Each routine restates what xtensor 0.27.1 executes for the call, in the
 * same loop order and arithmetic types, compiled -O2 with OpenMP over the
 * loops the reference parallelises (assignment: xassign.hpp:725-842,
 * 1148-1286) and — more generously than the reference, whose lazy reducers
 * are single-threaded — over independent reduction outputs:
 *
 *   bl_transpose_201_*  xt::xarray<T> t = xt::transpose(x, {2, 0, 1});
 *                       the stepper_assigner walks the destination in
 *                       row-major order reading the permuted source
 *                       (xassign.hpp:644-695, 1087, 1341).
 *   bl_normalize_*      (x - mean(x,{2},keep_dims)) / sqrt(variance(x,{2},keep_dims) + eps):
 *                       mean = sum in T (sequential) / (double)n
 *                       (xmath.hpp:1828-1858); variance = mean of
 *                       square(x - mean) in double (xmath.hpp:2082-2103);
 *                       the elementwise tree in double, stored as T.
 *   bl_amax_02_*        xt::amax(x, {0, 2}): per output, innermost axis folds
 *                       select(acc > v) from lowest(), outer axis merges
 *                       (xreducer.hpp:1801-1828, xmath.hpp:589-602, 777-793).
 *   bl_argmax_1_*       xt::argmax(x, 1): a transposed copy moving axis 1
 *                       last, then a strict-greater scan per row
 *                       (xsort.hpp:1158-1235).
 *   bl_c0_*             E = A * b + exp(-A * A); r = sum(E, {1}).
 *   bl_c3_rowsum_f32    one batching instance: r = sum(A * v + C, {1}).
 *   bl_sum_*            full sums (sequential, as the lazy reducer).
 *   bl_stat_*_f32 / _bf16
 *                       the precision workload's full reductions, one
 *                       sequential pass each as the lazy reducer runs them,
 *                       single-threaded (the reference's reducers are):
 *                       sum in the value type (bfloat16 values widen to
 *                       float, their sum type); mean = sum / (double)n
 *                       (xmath.hpp:1860-1872); variance = mean over
 *                       square(x - mean) with the double mean, summed in
 *                       double (xmath.hpp:2033-2037); norm_l2 = sqrt of the
 *                       double sum of x * x computed in the value type
 *                       (xnorm.hpp:397-437, norm_sq(t) = t * t).
 *   bl_cumsum_*         xt::cumsum(x, axis) on a contiguous (d0, d1, d2) array:
 *                       `res = x`, then res[.., i, ..] += res[.., i-1, ..]
 *                       walking the storage with the axis stride
 *                       (xaccumulator.hpp:233-281); axis = -1 flattens
 *                       (:283-310).  The copy is fused into the first pass.
 *   bl_blockwise_sum_axis0_f32 / bl_blockwise_mean_12_f32
 *                       xt::blockwise::sum(x, {b0, b1, b2}, {0}) and
 *                       blockwise::mean(x, blocks, {1, 2}) on a contiguous
 *                       (d0, d1, d2) float array: each block summed in the
 *                       plain reducer's order, block results folded in grid
 *                       order, the mean divided at the end
 *                       (xblockwise_reducer.hpp:129-194, functors :38-160);
 *                       OpenMP over independent outputs.
 *   bl_chunked_*        chunked arrays of rank 3: assignment chunk by chunk,
 *                       reading, and sum over the last axis (below).
 *   bl_npy_load         xt::load_npy<T>(filename): read the magic and version,
 *                       the header length and the header, take the word
 *                       size from 'descr' and the shape from 'shape', then
 *                       read the whole data block into one heap buffer with
 *                       one read (xnpy.hpp:674-705, 540-566).
 *   bl_npy_save         xt::dump_npy(filename, e) of an evaluated container:
 *                       write the header, then the data with one write
 *                       (xnpy.hpp:707-742).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define DEF_TRANSPOSE(T, NAME)                                                           \
    void bl_transpose_201_##NAME(const T* x, T* out, int64_t d0, int64_t d1, int64_t d2) { \
        _Pragma("omp parallel for schedule(static)")                                      \
        for (int64_t k = 0; k < d2; ++k) {                                                 \
            T* o = out + k * d0 * d1;                                                      \
            for (int64_t i = 0; i < d0; ++i)                                               \
                for (int64_t j = 0; j < d1; ++j) o[i * d1 + j] = x[(i * d1 + j) * d2 + k];  \
        }                                                                                  \
    }
DEF_TRANSPOSE(float, f32)
DEF_TRANSPOSE(double, f64)

#define DEF_NORMALIZE(T, NAME)                                                                   \
    void bl_normalize_##NAME(const T* x, T* y, int64_t rows, int64_t n, double eps) {            \
        _Pragma("omp parallel for schedule(static)")                                              \
        for (int64_t r = 0; r < rows; ++r) {                                                       \
            const T* xr = x + r * n;                                                               \
            T s = 0;                                                                               \
            for (int64_t k = 0; k < n; ++k) s = s + xr[k];                                         \
            double mean = (double)s / (double)n;                                                   \
            double q = 0;                                                                          \
            for (int64_t k = 0; k < n; ++k) {                                                      \
                double d = (double)xr[k] - mean;                                                   \
                q = q + d * d;                                                                     \
            }                                                                                      \
            double var = q / (double)n;                                                            \
            double den = sqrt(var + eps);                                                          \
            T* yr = y + r * n;                                                                     \
            for (int64_t k = 0; k < n; ++k) yr[k] = (T)(((double)xr[k] - mean) / den);             \
        }                                                                                          \
    }
DEF_NORMALIZE(float, f32)
DEF_NORMALIZE(double, f64)

#define DEF_AMAX(T, NAME, LOWEST)                                                        \
    void bl_amax_02_##NAME(const T* x, T* out, int64_t d0, int64_t d1, int64_t d2) {     \
        _Pragma("omp parallel for schedule(static)")                                      \
        for (int64_t j = 0; j < d1; ++j) {                                                 \
            T res = 0;                                                                     \
            for (int64_t i = 0; i < d0; ++i) {                                             \
                const T* row = x + (i * d1 + j) * d2;                                      \
                T acc = LOWEST;                                                            \
                for (int64_t k = 0; k < d2; ++k) acc = acc > row[k] ? acc : row[k];        \
                res = i == 0 ? acc : (res > acc ? res : acc);                              \
            }                                                                              \
            out[j] = res;                                                                  \
        }                                                                                  \
    }
DEF_AMAX(float, f32, -3.40282346638528859812e+38f)
DEF_AMAX(double, f64, -1.7976931348623157e+308)

#define DEF_ARGMAX(T, NAME)                                                                          \
    void bl_argmax_1_##NAME(const T* x, int32_t* out, int64_t d0, int64_t d1, int64_t d2, T* tmp) {  \
        /* eval_type input = transpose(e, {0, 2, 1}) */                                              \
        _Pragma("omp parallel for schedule(static)")                                                  \
        for (int64_t i = 0; i < d0; ++i)                                                               \
            for (int64_t k = 0; k < d2; ++k)                                                           \
                for (int64_t j = 0; j < d1; ++j) tmp[(i * d2 + k) * d1 + j] = x[(i * d1 + j) * d2 + k]; \
        _Pragma("omp parallel for schedule(static)")                                                  \
        for (int64_t r = 0; r < d0 * d2; ++r) {                                                        \
            const T* row = tmp + r * d1;                                                               \
            T v = row[0];                                                                              \
            int64_t idx = 0;                                                                           \
            for (int64_t j = 1; j < d1; ++j)                                                           \
                if (row[j] > v) {                                                                      \
                    v = row[j];                                                                        \
                    idx = j;                                                                           \
                }                                                                                      \
            out[r] = (int32_t)idx;                                                                     \
        }                                                                                              \
    }
DEF_ARGMAX(float, f32)
DEF_ARGMAX(double, f64)

void bl_c0_assign(const float* A, const float* b, float* E, int64_t n, int64_t m) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < m; ++j) {
            float a = A[i * m + j];
            E[i * m + j] = a * b[j] + expf(-a * a);
        }
}

void bl_c0_sum(const float* E, float* r, int64_t n, int64_t m) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float s = 0.f;
        for (int64_t j = 0; j < m; ++j) s = s + E[i * m + j];
        r[i] = s;
    }
}

/* C3, one instance: r = sum(A * v + C, {1}) with A, C (n, m) and v (m,)
 * float32: the lazy reducer evaluates the xfunction element by element in
 * float and folds each row sequentially in float (xreducer.hpp:1819-1825);
 * rows in parallel. */
void bl_c3_rowsum_f32(const float* A, const float* v, const float* Cm, float* r, int64_t n, int64_t m) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float s = 0.f;
        for (int64_t j = 0; j < m; ++j) s = s + (A[i * m + j] * v[j] + Cm[i * m + j]);
        r[i] = s;
    }
}

float bl_sum_f32(const float* x, int64_t n) {
    float s = 0.f;
    for (int64_t i = 0; i < n; ++i) s = s + x[i];
    return s;
}

int64_t bl_sum_i32_i64(const int32_t* x, int64_t n) {
    int64_t s = 0;
    for (int64_t i = 0; i < n; ++i) s += x[i];
    return s;
}

static inline float bl_bf16(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

#define DEF_STATS(NAME, T, LOAD)                                                     \
    float bl_stat_sum_##NAME(const T* x, int64_t n) {                                \
        float s = 0.f;                                                               \
        for (int64_t i = 0; i < n; ++i) s = s + LOAD(x[i]);                          \
        return s;                                                                    \
    }                                                                                \
    double bl_stat_mean_##NAME(const T* x, int64_t n) {                              \
        return n ? (double)bl_stat_sum_##NAME(x, n) / (double)n : 0.0;               \
    }                                                                                \
    double bl_stat_variance_##NAME(const T* x, int64_t n) {                          \
        const double m = bl_stat_mean_##NAME(x, n);                                  \
        double q = 0.0;                                                              \
        for (int64_t i = 0; i < n; ++i) {                                            \
            const double d = (double)LOAD(x[i]) - m;                                 \
            q = q + d * d;                                                           \
        }                                                                            \
        return n ? q / (double)n : 0.0;                                              \
    }                                                                                \
    double bl_stat_norm_l2_##NAME(const T* x, int64_t n) {                           \
        double q = 0.0;                                                              \
        for (int64_t i = 0; i < n; ++i) {                                            \
            const float v = LOAD(x[i]);                                              \
            q = q + (double)(v * v);                                                 \
        }                                                                            \
        return sqrt(q);                                                              \
    }
#define BL_ID(v) (v)
DEF_STATS(f32, float, BL_ID)
DEF_STATS(bf16, uint16_t, bl_bf16)


#define DEF_CUMSUM(T, NAME)                                                                           \
    void bl_cumsum_##NAME(const T* x, T* r, int64_t d0, int64_t d1, int64_t d2, int axis) {           \
        if (axis < 0) {                                                                               \
            const int64_t n = d0 * d1 * d2;                                                           \
            T acc = 0;                                                                                \
            for (int64_t i = 0; i < n; ++i) r[i] = acc = (i ? acc + x[i] : x[i]);                      \
            return;                                                                                   \
        }                                                                                             \
        const int64_t outer = axis == 0 ? 1 : (axis == 1 ? d0 : d0 * d1);                             \
        const int64_t len = axis == 0 ? d0 : (axis == 1 ? d1 : d2);                                   \
        const int64_t inner = axis == 0 ? d1 * d2 : (axis == 1 ? d2 : 1);                             \
        _Pragma("omp parallel for schedule(static)")                                                  \
        for (int64_t o = 0; o < outer; ++o) {                                                         \
            const T* xo = x + o * len * inner;                                                        \
            T* ro = r + o * len * inner;                                                              \
            for (int64_t j = 0; j < inner; ++j) ro[j] = xo[j];                                        \
            for (int64_t i = 1; i < len; ++i)                                                         \
                for (int64_t j = 0; j < inner; ++j) ro[i * inner + j] = ro[(i - 1) * inner + j] + xo[i * inner + j]; \
        }                                                                                             \
    }
DEF_CUMSUM(float, f32)
DEF_CUMSUM(double, f64)
DEF_CUMSUM(int32_t, i32)


/* Returns the data bytes read into *out (malloc'd; free with bl_free), -1 on error. */
int64_t bl_npy_load(const char* path, void** out) {
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    unsigned char pre[8];
    int64_t res = -1;
    char* header = NULL;
    if (fread(pre, 1, 8, f) != 8 || memcmp(pre, "\x93NUMPY", 6) != 0) goto done;
    unsigned char lb[4] = {0, 0, 0, 0};
    const size_t nl = pre[6] == 1 ? 2 : 4;
    if (fread(lb, 1, nl, f) != nl) goto done;
    const size_t hl = (size_t)lb[0] | (size_t)lb[1] << 8 | (size_t)lb[2] << 16 | (size_t)lb[3] << 24;
    header = (char*)malloc(hl + 1);
    if (!header || fread(header, 1, hl, f) != hl) goto done;
    header[hl] = 0;
    const char* d = strstr(header, "'descr'");
    const char* sh = strstr(header, "'shape'");
    if (!d || !sh) goto done;
    d = strchr(d + 7, '\'');
    if (!d) goto done;
    const int64_t word = strtoll(d + 3, NULL, 10);
    const char* p = strchr(sh, '(');
    if (!p) goto done;
    int64_t n = 1;
    for (++p; *p && *p != ')';) {
        char* e;
        const long long v = strtoll(p, &e, 10);
        if (e == p) {
            ++p;
            continue;
        }
        n *= v;
        p = e;
    }
    const int64_t bytes = n * word;
    void* buf = malloc(bytes > 0 ? (size_t)bytes : 1);
    if (!buf) goto done;
    if ((int64_t)fread(buf, 1, (size_t)bytes, f) != bytes) {
        free(buf);
        goto done;
    }
    *out = buf;
    res = bytes;
done:
    free(header);
    fclose(f);
    return res;
}

int bl_npy_save(const char* path, const void* header, int64_t hlen, const void* data, int64_t nbytes) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    int ok = fwrite(header, 1, (size_t)hlen, f) == (size_t)hlen && fwrite(data, 1, (size_t)nbytes, f) == (size_t)nbytes;
    ok = (fclose(f) == 0) && ok;
    return ok ? 0 : -1;
}

void bl_free(void* p) { free(p); }

void bl_blockwise_sum_axis0_f32(const float* x, float* out, int64_t d0, int64_t d1, int64_t d2, int64_t b0) {
    const int64_t m = d1 * d2;
    _Pragma("omp parallel for schedule(static)")
    for (int64_t j0 = 0; j0 < m; j0 += 4096) {
        const int64_t j1 = j0 + 4096 < m ? j0 + 4096 : m;
        float part[4096];
        for (int64_t i0 = 0; i0 < d0; i0 += b0) {
            const int64_t i1 = i0 + b0 < d0 ? i0 + b0 : d0;
            for (int64_t j = j0; j < j1; ++j) part[j - j0] = x[i0 * m + j];
            for (int64_t i = i0 + 1; i < i1; ++i)
                for (int64_t j = j0; j < j1; ++j) part[j - j0] += x[i * m + j];
            for (int64_t j = j0; j < j1; ++j) out[j] = i0 == 0 ? part[j - j0] : out[j] + part[j - j0];
        }
    }
}

void bl_blockwise_mean_12_f32(const float* x, double* out, int64_t d0, int64_t d1, int64_t d2, int64_t b1, int64_t b2) {
    _Pragma("omp parallel for schedule(static)")
    for (int64_t i = 0; i < d0; ++i) {
        const float* r = x + i * d1 * d2;
        double acc = 0;
        int first = 1;
        for (int64_t k0 = 0; k0 < d1; k0 += b1)
            for (int64_t l0 = 0; l0 < d2; l0 += b2) {
                const int64_t k1 = k0 + b1 < d1 ? k0 + b1 : d1, l1 = l0 + b2 < d2 ? l0 + b2 : d2;
                double s = 0;
                for (int64_t k = k0; k < k1; ++k)
                    for (int64_t l = l0; l < l1; ++l) s += r[k * d2 + l];
                acc = first ? s : acc + s;
                first = 0;
            }
        out[i] = acc / (double)(d1 * d2);
    }
}

/* Chunked arrays of rank 3 (shape d, chunk shape c, grid g = ceil(d / c)),
 * chunks row-major of c elements, given as an array of chunk pointers in the
 * grid's row-major order:
 *   bl_chunked_axpb_f32   a = x * s + t into the chunks, chunk by chunk in
 *                         grid order (xchunked_semantic::assign_xexpression,
 *                         chunk/xchunked_assign.hpp:200-219), each chunk's
 *                         valid region only; OpenMP over chunks;
 *   bl_chunked_read_f32   the dense array of a chunked one (reading it
 *                         element by element through the chunk index,
 *                         xchunked_array.hpp:440-460, 640-646);
 *   bl_chunked_sum2_f32   xt::sum(a, {2}): per output a sequential float fold
 *                         over the last axis through the chunk index (the
 *                         lazy reducer, xreducer.hpp:1801-1828); OpenMP over
 *                         outputs. */
static inline const float* bl_chunk_at(float* const* chunks, const int64_t* d, const int64_t* c, int64_t i, int64_t j,
                                       int64_t k) {
    const int64_t g1 = (d[1] + c[1] - 1) / c[1], g2 = (d[2] + c[2] - 1) / c[2];
    const int64_t ci = ((i / c[0]) * g1 + j / c[1]) * g2 + k / c[2];
    return chunks[ci] + ((i % c[0]) * c[1] + j % c[1]) * c[2] + k % c[2];
}

void bl_chunked_axpb_f32(const float* x, float* const* chunks, const int64_t* d, const int64_t* c, float s, float t) {
    const int64_t g0 = (d[0] + c[0] - 1) / c[0], g1 = (d[1] + c[1] - 1) / c[1], g2 = (d[2] + c[2] - 1) / c[2];
    _Pragma("omp parallel for schedule(dynamic)")
    for (int64_t ci = 0; ci < g0 * g1 * g2; ++ci) {
        const int64_t a = ci / (g1 * g2), b = (ci / g2) % g1, e = ci % g2;
        const int64_t e0 = d[0] - a * c[0] < c[0] ? d[0] - a * c[0] : c[0];
        const int64_t e1 = d[1] - b * c[1] < c[1] ? d[1] - b * c[1] : c[1];
        const int64_t e2 = d[2] - e * c[2] < c[2] ? d[2] - e * c[2] : c[2];
        float* ch = chunks[ci];
        for (int64_t i = 0; i < e0; ++i)
            for (int64_t j = 0; j < e1; ++j) {
                const float* xr = x + ((a * c[0] + i) * d[1] + b * c[1] + j) * d[2] + e * c[2];
                float* cr = ch + (i * c[1] + j) * c[2];
                for (int64_t k = 0; k < e2; ++k) cr[k] = xr[k] * s + t;
            }
    }
}

void bl_chunked_read_f32(float* const* chunks, float* out, const int64_t* d, const int64_t* c) {
    _Pragma("omp parallel for schedule(static)")
    for (int64_t i = 0; i < d[0]; ++i)
        for (int64_t j = 0; j < d[1]; ++j)
            for (int64_t k = 0; k < d[2]; ++k) out[(i * d[1] + j) * d[2] + k] = *bl_chunk_at(chunks, d, c, i, j, k);
}

void bl_chunked_sum2_f32(float* const* chunks, float* out, const int64_t* d, const int64_t* c) {
    _Pragma("omp parallel for schedule(static)")
    for (int64_t r = 0; r < d[0] * d[1]; ++r) {
        const int64_t i = r / d[1], j = r % d[1];
        float s = 0.f;
        for (int64_t k = 0; k < d[2]; ++k) s = s + *bl_chunk_at(chunks, d, c, i, j, k);
        out[r] = s;
    }
}
