/*
 * xt_oracle.c — CPU restatement of xtensor's assign + reduce semantics.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the parity oracle (and, for the
 * bench's CPU baseline, the timed CPU port).  The product library never
 * links, loads or calls it.
 *
 * The reference (xtensor 0.27.1) cannot be compiled here: it requires xtl
 * 0.8.0 (and xsimd for its SIMD path), neither of which is available.  This
 * file restates the reference's algorithms on the same C structs the GPU
 * library takes (include/xtg.h), with host pointers:
 *
 *   orc_assign     — element-by-element evaluation of the lowered xfunction
 *                    tree in C++ arithmetic (the scalar stepper_assigner,
 *                    include/xtensor/core/xassign.hpp:644-695, evaluating
 *                    xfunction_stepper::operator*, core/xfunction.hpp:1108-1118);
 *   orc_reduce     — xreducer_stepper::aggregate / aggregate_impl with the
 *                    reference's loop order: the innermost reduced axis folds
 *                    with `reduce` from init, outer reduced axes fold the
 *                    partial results with `merge`
 *                    (include/xtensor/reducers/xreducer.hpp:1778-1828);
 *                    mean = sum / (double)((size - ddof) / n_out)
 *                    (core/xmath.hpp:1828-1858); variance = mean of squared
 *                    deviations from the evaluated mean (core/xmath.hpp:2082-2103);
 *   orc_argreduce  — arg_func_impl: strict compare, first index wins
 *                    (include/xtensor/misc/xsort.hpp:1158-1296);
 *   orc_accumulate — accumulator_impl: conversion to the accumulation type,
 *                    then a sequential fold along the axis or over the
 *                    row-major flattening
 *                    (include/xtensor/reducers/xaccumulator.hpp:154-310).
 *
 * Arithmetic is carried out in the C type of each node (float ops in float,
 * integer ops wrapped to their width), with -ffp-contract=off so that no
 * multiply-add is fused.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xtg.h"

static __thread char g_err[512];
const char* orc_last_error(void) { return g_err; }
static int err(int code, const char* msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}

/* ---- dtypes ---------------------------------------------------------------- */
static const int DSIZE[XTG_NUM_DTYPES] = {1, 1, 1, 2, 2, 4, 4, 8, 8, 2, 4, 8};
static int is_float(int t) { return t == XTG_FLOAT32 || t == XTG_FLOAT64 || t == XTG_BFLOAT16; }
static int is_signed_int(int t) { return t == XTG_INT8 || t == XTG_INT16 || t == XTG_INT32 || t == XTG_INT64; }
static int valid(int t) { return t >= 0 && t < XTG_NUM_DTYPES; }

/* C++ integral promotion and usual arithmetic conversions (bf16 counts as a
 * narrow float promoted to float). */
static int iprom(int a) {
    if (a == XTG_BOOL || a == XTG_INT8 || a == XTG_UINT8 || a == XTG_INT16 || a == XTG_UINT16) return XTG_INT32;
    if (a == XTG_BFLOAT16) return XTG_FLOAT32;
    return a;
}
static int irank(int t) { return (t == XTG_INT64 || t == XTG_UINT64) ? 2 : 1; }
int orc_promote(int a, int b) {
    if (a == XTG_FLOAT64 || b == XTG_FLOAT64) return XTG_FLOAT64;
    if (a == XTG_FLOAT32 || b == XTG_FLOAT32 || a == XTG_BFLOAT16 || b == XTG_BFLOAT16) return XTG_FLOAT32;
    a = iprom(a);
    b = iprom(b);
    if (a == b) return a;
    int sa = is_signed_int(a), sb = is_signed_int(b);
    if (sa == sb) return irank(a) >= irank(b) ? a : b;
    int u = sa ? b : a, s = sa ? a : b;
    return irank(u) >= irank(s) ? u : s;
}

/* bf16 <-> float from the format definition (round to nearest even). */
static float bf16_to_f(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static uint16_t f_to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

/* A typed scalar value.  Floats keep their exact value in `f` (float values
 * are exactly representable in double); integers in `i` / `u`. */
typedef struct {
    int t;
    double f;
    int64_t i;
    uint64_t u;
} val;

static val mk_f(int t, double f) {
    val v;
    v.t = t;
    v.f = (t == XTG_FLOAT32) ? (double)(float)f : f;
    v.i = 0;
    v.u = 0;
    return v;
}
/* wrap an integer to type t (two's complement / unsigned modulo) */
static val mk_u(int t, uint64_t x) {
    val v;
    v.t = t;
    v.f = 0;
    switch (t) {
        case XTG_BOOL: x = x ? 1 : 0; v.i = (int64_t)x; break;
        case XTG_INT8: v.i = (int8_t)(uint8_t)x; break;
        case XTG_UINT8: v.i = (uint8_t)x; break;
        case XTG_INT16: v.i = (int16_t)(uint16_t)x; break;
        case XTG_UINT16: v.i = (uint16_t)x; break;
        case XTG_INT32: v.i = (int32_t)(uint32_t)x; break;
        case XTG_UINT32: v.i = (uint32_t)x; break;
        case XTG_INT64: v.i = (int64_t)x; break;
        default: v.i = (int64_t)x; break;
    }
    v.u = (t == XTG_UINT64) ? x : (uint64_t)v.i;
    return v;
}

/* static_cast<T>(v) */
static val cvt(val v, int t) {
    if (v.t == t) return v;
    if (t == XTG_BOOL) {
        int nz = is_float(v.t) ? (v.f != 0.0) : (v.u != 0);
        return mk_u(XTG_BOOL, (uint64_t)nz);
    }
    if (is_float(t)) {
        double x;
        if (is_float(v.t)) x = v.f;
        else if (v.t == XTG_UINT64) x = (double)v.u;
        else x = (double)v.i;
        if (t == XTG_FLOAT32) {
            float y;
            if (is_float(v.t)) y = (float)v.f;
            else if (v.t == XTG_UINT64) y = (float)v.u;
            else y = (float)v.i;
            return mk_f(XTG_FLOAT32, y);
        }
        if (t == XTG_BFLOAT16) return mk_f(XTG_BFLOAT16, bf16_to_f(f_to_bf16((float)x)));
        return mk_f(XTG_FLOAT64, x);
    }
    /* to integer */
    if (is_float(v.t)) {
        double x = v.f;
        if (t == XTG_UINT64) return mk_u(t, (uint64_t)x);
        if (t == XTG_UINT32) return mk_u(t, (uint64_t)(uint32_t)(int64_t)x);
        return mk_u(t, (uint64_t)(int64_t)x);
    }
    return mk_u(t, v.u);
}

static double as_d(val v) { return is_float(v.t) ? v.f : (v.t == XTG_UINT64 ? (double)v.u : (double)v.i); }

/* ---- expression tree --------------------------------------------------------- */
typedef struct {
    const xtg_expr* e;
    int kids[XTG_MAX_NODES][3];
    int nk[XTG_MAX_NODES];
    int type[XTG_MAX_NODES];
    int root;
    int rank;
    int64_t shape[XTG_MAX_RANK];
} otree;

static int arity(int op) {
    if (op == XTG_OP_LEAF || op == XTG_OP_SCALAR) return 0;
    if (op >= XTG_OP_NEG && op <= XTG_OP_CAST) return 1;
    if (op >= XTG_OP_ADD && op <= XTG_OP_POW) return 2;
    if (op == XTG_OP_WHERE) return 3;
    if (op >= XTG_OP_RSUM && op <= XTG_OP_RMIN) return 1;
    return -1;
}

static int fn_type(int a) { return (a == XTG_FLOAT32 || a == XTG_BFLOAT16) ? XTG_FLOAT32 : XTG_FLOAT64; }

static int node_type(otree* T, int n) {
    const xtg_node* x = &T->e->nodes[n];
    int a = T->nk[n] > 0 ? T->type[T->kids[n][0]] : -1;
    int b = T->nk[n] > 1 ? T->type[T->kids[n][1]] : -1;
    switch (x->op) {
        case XTG_OP_LEAF: return T->e->leaves[x->arg].dtype;
        case XTG_OP_SCALAR: return x->dtype;
        case XTG_OP_CAST: return x->arg;
        case XTG_OP_NEG:
        case XTG_OP_POS:
        case XTG_OP_BIT_NOT: return iprom(a);
        case XTG_OP_SQUARE: return orc_promote(a, a);
        case XTG_OP_ABS: return (a == XTG_UINT32 || a == XTG_UINT64) ? a : iprom(a);
        case XTG_OP_EXP:
        case XTG_OP_LOG:
        case XTG_OP_SQRT:
        case XTG_OP_SIN:
        case XTG_OP_COS:
        case XTG_OP_TANH: return fn_type(a);
        case XTG_OP_LOGICAL_NOT: return XTG_BOOL;
        case XTG_OP_POW: return (is_float(a) && is_float(b) && fn_type(a) == XTG_FLOAT32 && fn_type(b) == XTG_FLOAT32) ? XTG_FLOAT32 : XTG_FLOAT64;
        case XTG_OP_WHERE: return orc_promote(b, T->type[T->kids[n][2]]);
        case XTG_OP_RSUM: return orc_promote(a, a);
        case XTG_OP_RMEAN:
        case XTG_OP_RVAR:
        case XTG_OP_RSTD: return XTG_FLOAT64;
        case XTG_OP_RMAX:
        case XTG_OP_RMIN: return a == XTG_BFLOAT16 ? XTG_FLOAT32 : a;
    }
    if (x->op >= XTG_OP_LT && x->op <= XTG_OP_LOGICAL_OR) return XTG_BOOL;
    return orc_promote(a, b);
}

static int build(const xtg_expr* e, otree* T) {
    memset(T, 0, sizeof *T);
    T->e = e;
    int st[XTG_MAX_NODES], sp = 0;
    if (e->n_nodes <= 0 || e->n_nodes > XTG_MAX_NODES) return err(XTG_ERR_INVALID, "bad node count");
    for (int i = 0; i < e->n_nodes; ++i) {
        int ar = arity(e->nodes[i].op);
        if (ar < 0) return err(XTG_ERR_INVALID, "unknown opcode");
        if (sp < ar) return err(XTG_ERR_INVALID, "stack underflow");
        T->nk[i] = ar;
        for (int k = 0; k < ar; ++k) T->kids[i][k] = st[sp - ar + k];
        sp -= ar;
        if (e->nodes[i].op == XTG_OP_LEAF && (e->nodes[i].arg < 0 || e->nodes[i].arg >= e->n_leaves))
            return err(XTG_ERR_INVALID, "leaf index");
        T->type[i] = node_type(T, i);
        st[sp++] = i;
    }
    if (sp != 1) return err(XTG_ERR_INVALID, "malformed postfix");
    T->root = st[0];
    /* broadcast shape over the leaves that are referenced */
    int used[XTG_MAX_LEAVES] = {0};
    for (int i = 0; i < e->n_nodes; ++i)
        if (e->nodes[i].op == XTG_OP_LEAF) used[e->nodes[i].arg] = 1;
    int rank = 0;
    for (int l = 0; l < e->n_leaves; ++l)
        if (used[l] && e->leaves[l].rank > rank) rank = e->leaves[l].rank;
    for (int d = 0; d < rank; ++d) T->shape[d] = 1;
    for (int l = 0; l < e->n_leaves; ++l) {
        if (!used[l]) continue;
        const xtg_array* a = &e->leaves[l];
        for (int i = 0; i < a->rank; ++i) {
            int d = rank - a->rank + i;
            if (T->shape[d] == 1) T->shape[d] = a->shape[i];
            else if (a->shape[i] != 1 && a->shape[i] != T->shape[d]) return err(XTG_ERR_BROADCAST, "broadcast");
        }
    }
    T->rank = rank;
    return 0;
}

static val load(const xtg_array* a, int64_t off) {
    const char* p = (const char*)a->data + off * DSIZE[a->dtype];
    switch (a->dtype) {
        case XTG_BOOL: return mk_u(XTG_BOOL, *(const uint8_t*)p);
        case XTG_INT8: return mk_u(XTG_INT8, (uint64_t)(int64_t) * (const int8_t*)p);
        case XTG_UINT8: return mk_u(XTG_UINT8, *(const uint8_t*)p);
        case XTG_INT16: return mk_u(XTG_INT16, (uint64_t)(int64_t) * (const int16_t*)p);
        case XTG_UINT16: return mk_u(XTG_UINT16, *(const uint16_t*)p);
        case XTG_INT32: return mk_u(XTG_INT32, (uint64_t)(int64_t) * (const int32_t*)p);
        case XTG_UINT32: return mk_u(XTG_UINT32, *(const uint32_t*)p);
        case XTG_INT64: return mk_u(XTG_INT64, (uint64_t) * (const int64_t*)p);
        case XTG_UINT64: return mk_u(XTG_UINT64, *(const uint64_t*)p);
        case XTG_BFLOAT16: return mk_f(XTG_BFLOAT16, bf16_to_f(*(const uint16_t*)p));
        case XTG_FLOAT32: return mk_f(XTG_FLOAT32, *(const float*)p);
        default: return mk_f(XTG_FLOAT64, *(const double*)p);
    }
}

static void store(const xtg_array* a, int64_t off, val v) {
    char* p = (char*)a->data + off * DSIZE[a->dtype];
    v = cvt(v, a->dtype);
    switch (a->dtype) {
        case XTG_BOOL: *(uint8_t*)p = (uint8_t)(v.i != 0); break;
        case XTG_INT8: *(int8_t*)p = (int8_t)v.i; break;
        case XTG_UINT8: *(uint8_t*)p = (uint8_t)v.i; break;
        case XTG_INT16: *(int16_t*)p = (int16_t)v.i; break;
        case XTG_UINT16: *(uint16_t*)p = (uint16_t)v.i; break;
        case XTG_INT32: *(int32_t*)p = (int32_t)v.i; break;
        case XTG_UINT32: *(uint32_t*)p = (uint32_t)v.i; break;
        case XTG_INT64: *(int64_t*)p = v.i; break;
        case XTG_UINT64: *(uint64_t*)p = v.u; break;
        case XTG_BFLOAT16: *(uint16_t*)p = f_to_bf16((float)v.f); break;
        case XTG_FLOAT32: *(float*)p = (float)v.f; break;
        default: *(double*)p = v.f; break;
    }
}

/* leaf offset at a multi-index of the tree shape (broadcast: size-1 or
 * missing dims do not move, xiterator.hpp:488-497) */
static int64_t leaf_off(const otree* T, const xtg_array* a, const int64_t* idx) {
    int64_t o = 0;
    for (int i = 0; i < a->rank; ++i) {
        int d = T->rank - a->rank + i;
        if (a->shape[i] != 1) o += idx[d] * a->strides[i];
    }
    return o;
}

/* ---- binary/unary arithmetic in type t ---------------------------------------------- */
static val arith(int op, int t, val a, val b) {
    a = cvt(a, t);
    b = cvt(b, t);
    if (t == XTG_FLOAT32) {
        float x = (float)a.f, y = (float)b.f, r = 0.f;
        switch (op) {
            case XTG_OP_ADD: r = x + y; break;
            case XTG_OP_SUB: r = x - y; break;
            case XTG_OP_MUL: r = x * y; break;
            case XTG_OP_DIV: r = x / y; break;
            case XTG_OP_MAXIMUM: r = x > y ? x : y; break;
            case XTG_OP_MINIMUM: r = x < y ? x : y; break;
            case XTG_OP_POW: r = powf(x, y); break;
        }
        return mk_f(t, r);
    }
    if (t == XTG_FLOAT64) {
        double x = a.f, y = b.f, r = 0;
        switch (op) {
            case XTG_OP_ADD: r = x + y; break;
            case XTG_OP_SUB: r = x - y; break;
            case XTG_OP_MUL: r = x * y; break;
            case XTG_OP_DIV: r = x / y; break;
            case XTG_OP_MAXIMUM: r = x > y ? x : y; break;
            case XTG_OP_MINIMUM: r = x < y ? x : y; break;
            case XTG_OP_POW: r = pow(x, y); break;
        }
        return mk_f(t, r);
    }
    /* integers: compute in 64 bits, wrap to the type */
    int sgn = is_signed_int(t);
    uint64_t x = a.u, y = b.u, r = 0;
    int64_t xs = a.i, ys = b.i;
    switch (op) {
        case XTG_OP_ADD: r = x + y; break;
        case XTG_OP_SUB: r = x - y; break;
        case XTG_OP_MUL: r = x * y; break;
        case XTG_OP_DIV: r = y ? (sgn ? (uint64_t)(xs / ys) : (t == XTG_UINT64 ? x / y : (uint64_t)(a.i / b.i))) : 0; break;
        case XTG_OP_MOD: r = y ? (sgn ? (uint64_t)(xs % ys) : (t == XTG_UINT64 ? x % y : (uint64_t)(a.i % b.i))) : 0; break;
        case XTG_OP_MAXIMUM: r = (sgn ? xs > ys : (t == XTG_UINT64 ? x > y : a.i > b.i)) ? x : y; break;
        case XTG_OP_MINIMUM: r = (sgn ? xs < ys : (t == XTG_UINT64 ? x < y : a.i < b.i)) ? x : y; break;
        case XTG_OP_BIT_AND: r = x & y; break;
        case XTG_OP_BIT_OR: r = x | y; break;
        case XTG_OP_BIT_XOR: r = x ^ y; break;
    }
    return mk_u(t, r);
}

static int cmp(int op, int t, val a, val b) {
    a = cvt(a, t);
    b = cvt(b, t);
    if (is_float(t)) {
        double x = a.f, y = b.f;
        switch (op) {
            case XTG_OP_LT: return x < y;
            case XTG_OP_LE: return x <= y;
            case XTG_OP_GT: return x > y;
            case XTG_OP_GE: return x >= y;
            case XTG_OP_EQ: return x == y;
            case XTG_OP_NE: return x != y;
        }
    } else if (t == XTG_UINT64) {
        uint64_t x = a.u, y = b.u;
        switch (op) {
            case XTG_OP_LT: return x < y;
            case XTG_OP_LE: return x <= y;
            case XTG_OP_GT: return x > y;
            case XTG_OP_GE: return x >= y;
            case XTG_OP_EQ: return x == y;
            case XTG_OP_NE: return x != y;
        }
    } else {
        int64_t x = a.i, y = b.i;
        switch (op) {
            case XTG_OP_LT: return x < y;
            case XTG_OP_LE: return x <= y;
            case XTG_OP_GT: return x > y;
            case XTG_OP_GE: return x >= y;
            case XTG_OP_EQ: return x == y;
            case XTG_OP_NE: return x != y;
        }
    }
    return 0;
}

typedef struct {
    double stat[XTG_MAX_NODES]; /* per R-node row statistic at the current row */
} rowctx;

static val eval(const otree* T, int n, const int64_t* idx, const rowctx* rc) {
    const xtg_node* x = &T->e->nodes[n];
    int t = T->type[n];
    switch (x->op) {
        case XTG_OP_LEAF: {
            const xtg_array* a = &T->e->leaves[x->arg];
            return load(a, leaf_off(T, a, idx));
        }
        case XTG_OP_SCALAR:
            if (is_float(t)) return mk_f(t, t == XTG_BFLOAT16 ? bf16_to_f(f_to_bf16((float)x->imm.f)) : x->imm.f);
            return mk_u(t, x->imm.u);
        default: break;
    }
    if (x->op >= XTG_OP_RSUM && x->op <= XTG_OP_RMIN) return cvt(mk_f(XTG_FLOAT64, rc->stat[n]), t);
    val a = eval(T, T->kids[n][0], idx, rc);
    switch (x->op) {
        case XTG_OP_NEG: {
            val c = cvt(a, t);
            if (t == XTG_FLOAT32) return mk_f(t, -(float)c.f);
            if (is_float(t)) return mk_f(t, -c.f);
            return mk_u(t, (uint64_t)0 - c.u);
        }
        case XTG_OP_POS: return cvt(a, t);
        case XTG_OP_CAST: return cvt(a, t);
        case XTG_OP_SQUARE: return arith(XTG_OP_MUL, t, a, a);
        case XTG_OP_LOGICAL_NOT: return mk_u(XTG_BOOL, !cvt(a, XTG_BOOL).i);
        case XTG_OP_BIT_NOT: return mk_u(t, ~cvt(a, t).u);
        case XTG_OP_ABS: {
            val c = cvt(a, t);
            if (t == XTG_FLOAT32) return mk_f(t, fabsf((float)c.f));
            if (is_float(t)) return mk_f(t, fabs(c.f));
            if (is_signed_int(t)) return mk_u(t, c.i < 0 ? (uint64_t)0 - c.u : c.u);
            return c;
        }
        case XTG_OP_EXP:
        case XTG_OP_LOG:
        case XTG_OP_SQRT:
        case XTG_OP_SIN:
        case XTG_OP_COS:
        case XTG_OP_TANH: {
            val c = cvt(a, t);
            if (t == XTG_FLOAT32) {
                float f = (float)c.f, r = 0;
                switch (x->op) {
                    case XTG_OP_EXP: r = expf(f); break;
                    case XTG_OP_LOG: r = logf(f); break;
                    case XTG_OP_SQRT: r = sqrtf(f); break;
                    case XTG_OP_SIN: r = sinf(f); break;
                    case XTG_OP_COS: r = cosf(f); break;
                    default: r = tanhf(f); break;
                }
                return mk_f(t, r);
            }
            double f = c.f, r = 0;
            switch (x->op) {
                case XTG_OP_EXP: r = exp(f); break;
                case XTG_OP_LOG: r = log(f); break;
                case XTG_OP_SQRT: r = sqrt(f); break;
                case XTG_OP_SIN: r = sin(f); break;
                case XTG_OP_COS: r = cos(f); break;
                default: r = tanh(f); break;
            }
            return mk_f(t, r);
        }
        default: break;
    }
    if (x->op == XTG_OP_WHERE) {
        int c = cvt(a, XTG_BOOL).i != 0;
        val b = eval(T, T->kids[n][1], idx, rc), d = eval(T, T->kids[n][2], idx, rc);
        return cvt(c ? b : d, t);
    }
    val b = eval(T, T->kids[n][1], idx, rc);
    if (x->op == XTG_OP_LOGICAL_AND) return mk_u(XTG_BOOL, cvt(a, XTG_BOOL).i && cvt(b, XTG_BOOL).i);
    if (x->op == XTG_OP_LOGICAL_OR) return mk_u(XTG_BOOL, cvt(a, XTG_BOOL).i || cvt(b, XTG_BOOL).i);
    if (x->op >= XTG_OP_LT && x->op <= XTG_OP_NE) return mk_u(XTG_BOOL, (uint64_t)cmp(x->op, orc_promote(a.t, b.t), a, b));
    return arith(x->op, t, a, b);
}

static void unflat(int64_t i, int rank, const int64_t* shape, int64_t* idx) {
    for (int d = rank - 1; d >= 0; --d) {
        idx[d] = shape[d] ? i % shape[d] : 0;
        i = shape[d] ? i / shape[d] : 0;
    }
}

/* Row statistics of every R node for the row at outer index `idx` (the last
 * `k` dims are the row): the reference evaluates mean/variance with keep_dims
 * as separate reductions, mean in the sum type then divided in double, and
 * variance as the mean of square(x - mean). */
static void row_stats(const otree* T, int64_t* idx, rowctx* rc) {
    const xtg_expr* e = T->e;
    for (int n = 0; n < e->n_nodes; ++n) {
        int op = e->nodes[n].op;
        if (op < XTG_OP_RSUM || op > XTG_OP_RMIN) continue;
        int k = e->nodes[n].arg;
        int64_t len = 1;
        for (int d = T->rank - k; d < T->rank; ++d) len *= T->shape[d];
        int64_t save[XTG_MAX_RANK];
        memcpy(save, idx, sizeof save);
        int sub = T->kids[n][0];
        int st = T->type[sub];
        int acct = orc_promote(st, st);
        val s = cvt(mk_u(XTG_INT32, 0), acct);
        double mx = 0;
        int have = 0;
        for (int64_t r = 0; r < len; ++r) {
            unflat(r, k, T->shape + T->rank - k, idx + T->rank - k);
            val v = eval(T, sub, idx, rc);
            if (op == XTG_OP_RMAX || op == XTG_OP_RMIN) {
                double dv = as_d(v);
                if (!have) { mx = dv; have = 1; }
                else if (op == XTG_OP_RMAX ? !(mx > dv) : !(mx < dv)) mx = dv;
            } else {
                s = arith(XTG_OP_ADD, acct, s, v);
            }
        }
        double sum = as_d(s);
        double mean = len ? sum / (double)len : NAN;
        double out = sum;
        if (op == XTG_OP_RMEAN) out = mean;
        if (op == XTG_OP_RMAX || op == XTG_OP_RMIN) out = mx;
        if (op == XTG_OP_RVAR || op == XTG_OP_RSTD) {
            double q = 0;
            for (int64_t r = 0; r < len; ++r) {
                unflat(r, k, T->shape + T->rank - k, idx + T->rank - k);
                double dv = as_d(eval(T, sub, idx, rc)) - mean;
                q += dv * dv;
            }
            int64_t nrows = 1;
            for (int d = 0; d < T->rank - k; ++d) nrows *= T->shape[d];
            int64_t div = nrows ? (nrows * len - e->nodes[n].aux) / nrows : 0;
            out = q / (double)div;
            if (op == XTG_OP_RSTD) out = sqrt(out);
        }
        rc->stat[n] = out;
        memcpy(idx, save, sizeof save);
    }
}

int orc_expr_dtype(const xtg_expr* e) {
    otree T;
    int s = build(e, &T);
    if (s) return -1;
    return T.type[T.root];
}

int orc_broadcast_shape(const xtg_expr* e, int32_t* rank, int64_t* shape) {
    otree T;
    int s = build(e, &T);
    if (s) return s;
    *rank = T.rank;
    for (int d = 0; d < T.rank; ++d) shape[d] = T.shape[d];
    return 0;
}

/* out = expression, element by element in row-major order of out. */
int orc_assign(const xtg_expr* e, const xtg_array* out) {
    static otree T;
    int s = build(e, &T);
    if (s) return s;
    int R = out->rank;
    if (T.rank > R) return err(XTG_ERR_SHAPE, "rank");
    /* evaluate against the destination's shape (broadcast of the tree) */
    otree U = T;
    U.rank = R;
    for (int d = 0; d < R; ++d) U.shape[d] = out->shape[d];
    int64_t n = 1;
    for (int d = 0; d < R; ++d) n *= out->shape[d];
    int has_r = 0, k = 0;
    for (int i = 0; i < e->n_nodes; ++i)
        if (e->nodes[i].op >= XTG_OP_RSUM && e->nodes[i].op <= XTG_OP_RMIN) has_r = 1, k = e->nodes[i].arg;
    if (has_r) {
        int64_t len = 1;
        for (int d = R - k; d < R; ++d) len *= out->shape[d];
        int64_t nrows = len ? n / len : 0;
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t r = 0; r < nrows; ++r) {
            int64_t idx[XTG_MAX_RANK] = {0};
            rowctx rc;
            unflat(r, R - k, out->shape, idx);
            row_stats(&U, idx, &rc);
            for (int64_t j = 0; j < len; ++j) {
                unflat(j, k, out->shape + R - k, idx + R - k);
                int64_t o = 0;
                for (int d = 0; d < R; ++d) o += idx[d] * out->strides[d];
                store(out, o, eval(&U, U.root, idx, &rc));
            }
        }
        return 0;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t idx[XTG_MAX_RANK];
        unflat(i, R, out->shape, idx);
        int64_t o = 0;
        for (int d = 0; d < R; ++d) o += idx[d] * out->strides[d];
        rowctx rc;
        store(out, o, eval(&U, U.root, idx, &rc));
    }
    return 0;
}

/* ---- reductions ------------------------------------------------------------------- */
static int big_promote(int t) {
    if (is_float(t)) return XTG_FLOAT64;
    return is_signed_int(t) ? XTG_INT64 : XTG_UINT64;
}

int orc_reduce_result_dtype(const xtg_expr* e, const xtg_reduce_desc* rd) {
    otree T;
    if (build(e, &T)) return -1;
    int vt = T.type[T.root];
    int init = (rd->acc_dtype >= 0 && valid(rd->acc_dtype)) ? rd->acc_dtype : vt;
    switch (rd->op) {
        case XTG_RED_SUM:
        case XTG_RED_PROD: return orc_promote(init, vt);
        case XTG_RED_AMAX:
        case XTG_RED_AMIN: return rd->acc_dtype >= 0 ? orc_promote(rd->acc_dtype, vt) : vt;
        case XTG_RED_MEAN:
        case XTG_RED_VARIANCE:
        case XTG_RED_STDDEV: return rd->acc_dtype >= 0 ? rd->acc_dtype : XTG_FLOAT64;
        case XTG_RED_NORM_L0: return XTG_UINT64;
        case XTG_RED_NORM_L1:
        case XTG_RED_NORM_SQ: return big_promote(vt);
        case XTG_RED_NORM_L2: return XTG_FLOAT64;
        case XTG_RED_NORM_LINF: {
            int a = vt == XTG_BFLOAT16 ? XTG_FLOAT32 : vt;
            return (a == XTG_UINT32 || a == XTG_UINT64 || is_float(a)) ? a : orc_promote(a, a);
        }
    }
    return -1;
}

typedef struct {
    const otree* T;
    int op;       /* reduce functor */
    int acct;     /* accumulator / result type */
    int nred;
    int red[XTG_MAX_RANK];
    val init;
    const double* mean_at; /* variance: per-output evaluated mean (NULL otherwise) */
    int64_t out_i;
} redctx;

/* value fed to the reduce functor at a full multi-index */
static val red_input(const redctx* c, const int64_t* idx) {
    rowctx rc;
    val v = eval(c->T, c->T->root, idx, &rc);
    switch (c->op) {
        case XTG_RED_VARIANCE:
        case XTG_RED_STDDEV: {
            double d = as_d(v) - c->mean_at[c->out_i];
            return mk_f(XTG_FLOAT64, d * d);
        }
        case XTG_RED_NORM_L0: {
            int nz = is_float(v.t) ? v.f != 0.0 : v.u != 0;
            return mk_u(XTG_UINT64, (uint64_t)nz);
        }
        case XTG_RED_NORM_L1:
        case XTG_RED_NORM_LINF: {
            int t = iprom(v.t);
            if (v.t == XTG_UINT32 || v.t == XTG_UINT64) return v;
            val c2 = cvt(v, t);
            if (t == XTG_FLOAT32) return mk_f(t, fabsf((float)c2.f));
            if (is_float(t)) return mk_f(t, fabs(c2.f));
            return mk_u(t, c2.i < 0 ? (uint64_t)0 - c2.u : c2.u);
        }
        case XTG_RED_NORM_SQ:
        case XTG_RED_NORM_L2: {
            int t = iprom(v.t);
            return arith(XTG_OP_MUL, t, v, v);
        }
    }
    return v;
}

static val fold(const redctx* c, val acc, val x) {
    switch (c->op) {
        case XTG_RED_PROD: return arith(XTG_OP_MUL, c->acct, acc, x);
        case XTG_RED_AMAX: {
            val xx = cvt(x, c->acct);
            return cmp(XTG_OP_GT, c->acct, acc, xx) ? acc : xx; /* select(t1 > t2, t1, t2) */
        }
        case XTG_RED_AMIN: {
            val xx = cvt(x, c->acct);
            return cmp(XTG_OP_LT, c->acct, acc, xx) ? acc : xx;
        }
        case XTG_RED_NORM_LINF: {
            val xx = cvt(x, c->acct);
            return cmp(XTG_OP_LT, c->acct, acc, xx) ? xx : acc; /* std::max(r, v) */
        }
    }
    return arith(XTG_OP_ADD, c->acct, acc, x);
}
static val merge(const redctx* c, val a, val b) {
    if (c->op == XTG_RED_NORM_LINF) return cmp(XTG_OP_GT, c->acct, a, b) ? a : b; /* math::maximum */
    return fold(c, a, b);
}

/* aggregate_impl(dim): recursive over the reduced axes (keep order). */
static val aggregate(const redctx* c, int dim, int64_t* idx) {
    int ax = c->red[dim];
    int64_t size = c->T->shape[ax];
    val res;
    if (dim != c->nred - 1) {
        idx[ax] = 0;
        res = aggregate(c, dim + 1, idx);
        for (int64_t i = 1; i < size; ++i) {
            idx[ax] = i;
            res = merge(c, res, aggregate(c, dim + 1, idx));
        }
    } else {
        idx[ax] = 0;
        res = fold(c, c->init, red_input(c, idx));
        for (int64_t i = 1; i < size; ++i) {
            idx[ax] = i;
            res = fold(c, res, red_input(c, idx));
        }
    }
    idx[ax] = 0;
    return res;
}

static int norm_axes(const xtg_reduce_desc* rd, int rank, int* axes, int* na) {
    if (rd->n_axes < 0) {
        for (int d = 0; d < rank; ++d) axes[d] = d;
        *na = rank;
        return 0;
    }
    *na = rd->n_axes;
    for (int i = 0; i < rd->n_axes; ++i) {
        int64_t a = rd->axes[i];
        if (a < 0) {
            a += rank;
            if (a < 0) return err(XTG_ERR_OUT_OF_RANGE, "axis out of range");
        }
        axes[i] = (int)a;
    }
    for (int i = 1; i < *na; ++i)
        if (axes[i] < axes[i - 1]) return err(XTG_ERR_AXIS, "Reducing axes should be sorted.");
    for (int i = 1; i < *na; ++i)
        if (axes[i] == axes[i - 1]) return err(XTG_ERR_AXIS, "Reducing axes should not contain duplicates.");
    if (*na && axes[*na - 1] > rank - 1) return err(XTG_ERR_AXIS, "Axis out of bounds for reduction.");
    return 0;
}

static val lowest_of(int t) {
    switch (t) {
        case XTG_FLOAT32: return mk_f(t, -3.40282346638528859812e+38);
        case XTG_FLOAT64: return mk_f(t, -1.7976931348623157e+308);
        case XTG_INT8: return mk_u(t, (uint64_t)(int64_t)-128);
        case XTG_INT16: return mk_u(t, (uint64_t)(int64_t)-32768);
        case XTG_INT32: return mk_u(t, (uint64_t)(int64_t)INT32_MIN);
        case XTG_INT64: return mk_u(t, (uint64_t)INT64_MIN);
        default: return mk_u(t, 0);
    }
}
static val max_of(int t) {
    switch (t) {
        case XTG_FLOAT32: return mk_f(t, 3.40282346638528859812e+38);
        case XTG_FLOAT64: return mk_f(t, 1.7976931348623157e+308);
        case XTG_BOOL: return mk_u(t, 1);
        case XTG_INT8: return mk_u(t, 127);
        case XTG_UINT8: return mk_u(t, 255);
        case XTG_INT16: return mk_u(t, 32767);
        case XTG_UINT16: return mk_u(t, 65535);
        case XTG_INT32: return mk_u(t, INT32_MAX);
        case XTG_UINT32: return mk_u(t, UINT32_MAX);
        case XTG_INT64: return mk_u(t, INT64_MAX);
        default: return mk_u(t, UINT64_MAX);
    }
}

static int reduce_pass(const otree* T, int op, int acct, const int* red, int nred, const int* kept, int nk,
                       val init, const double* mean_at, val* res, int64_t n_out) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t o = 0; o < n_out; ++o) {
        redctx c;
        c.T = T;
        c.op = op;
        c.acct = acct;
        c.nred = nred;
        memcpy(c.red, red, sizeof(int) * XTG_MAX_RANK);
        c.init = init;
        c.mean_at = mean_at;
        c.out_i = o;
        int64_t idx[XTG_MAX_RANK] = {0};
        int64_t kshape[XTG_MAX_RANK], kidx[XTG_MAX_RANK];
        for (int i = 0; i < nk; ++i) kshape[i] = T->shape[kept[i]];
        unflat(o, nk, kshape, kidx);
        for (int i = 0; i < nk; ++i) idx[kept[i]] = kidx[i];
        int64_t nel = 1;
        for (int i = 0; i < nred; ++i) nel *= T->shape[red[i]];
        if (nel == 0) res[o] = init;
        else if (nred == 0) res[o] = fold(&c, init, red_input(&c, idx));
        else res[o] = aggregate(&c, 0, idx);
    }
    return 0;
}

int orc_reduce(const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* out) {
    static otree T;
    int s = build(e, &T);
    if (s) return s;
    int axes[XTG_MAX_RANK], na;
    s = norm_axes(rd, T.rank, axes, &na);
    if (s) return s;
    int isred[XTG_MAX_RANK] = {0};
    for (int i = 0; i < na; ++i) isred[axes[i]] = 1;
    int kept[XTG_MAX_RANK], nk = 0;
    for (int d = 0; d < T.rank; ++d)
        if (!isred[d]) kept[nk++] = d;
    int64_t n_out = 1, size = 1;
    for (int i = 0; i < nk; ++i) n_out *= T.shape[kept[i]];
    for (int d = 0; d < T.rank; ++d) size *= T.shape[d];
    int vt = T.type[T.root];
    int rt = orc_reduce_result_dtype(e, rd);
    if (out->dtype != rt) return err(XTG_ERR_INVALID, "destination dtype");
    val* res = (val*)malloc(sizeof(val) * (n_out ? n_out : 1));
    double* mean_at = NULL;
    int op = rd->op;
    int init_t = (rd->acc_dtype >= 0) ? rd->acc_dtype : vt;
    int sumt = orc_promote(init_t, vt);
    if (op == XTG_RED_SUM || op == XTG_RED_MEAN) {
        reduce_pass(&T, XTG_RED_SUM, sumt, axes, na, kept, nk, cvt(mk_u(XTG_INT32, 0), sumt), NULL, res, n_out);
    } else if (op == XTG_RED_PROD) {
        reduce_pass(&T, op, sumt, axes, na, kept, nk, cvt(mk_u(XTG_INT32, 1), sumt), NULL, res, n_out);
    } else if (op == XTG_RED_AMAX || op == XTG_RED_AMIN) {
        int at = rt == XTG_BFLOAT16 ? XTG_FLOAT32 : rt;
        reduce_pass(&T, op, at, axes, na, kept, nk, op == XTG_RED_AMAX ? lowest_of(at) : max_of(at), NULL, res, n_out);
    } else if (op == XTG_RED_VARIANCE || op == XTG_RED_STDDEV) {
        /* inner_mean = eval(mean(x, axes, immediate)) */
        val* m = (val*)malloc(sizeof(val) * (n_out ? n_out : 1));
        int st = orc_promote(vt, vt);
        reduce_pass(&T, XTG_RED_SUM, st, axes, na, kept, nk, cvt(mk_u(XTG_INT32, 0), st), NULL, m, n_out);
        mean_at = (double*)malloc(sizeof(double) * (n_out ? n_out : 1));
        double mdiv = n_out ? (double)(size / n_out) : 0.0;
        for (int64_t o = 0; o < n_out; ++o) mean_at[o] = as_d(m[o]) / mdiv;
        free(m);
        reduce_pass(&T, op, XTG_FLOAT64, axes, na, kept, nk, mk_f(XTG_FLOAT64, 0.0), mean_at, res, n_out);
    } else if (op == XTG_RED_NORM_L0) {
        reduce_pass(&T, op, XTG_UINT64, axes, na, kept, nk, mk_u(XTG_UINT64, 0), NULL, res, n_out);
    } else if (op == XTG_RED_NORM_L1 || op == XTG_RED_NORM_SQ || op == XTG_RED_NORM_L2) {
        int bt = big_promote(vt);
        reduce_pass(&T, op, bt, axes, na, kept, nk, cvt(mk_u(XTG_INT32, 0), bt), NULL, res, n_out);
    } else if (op == XTG_RED_NORM_LINF) {
        reduce_pass(&T, op, rt, axes, na, kept, nk, cvt(mk_u(XTG_INT32, 0), rt), NULL, res, n_out);
    } else {
        free(res);
        return err(XTG_ERR_INVALID, "unknown reduction");
    }
    int64_t ddof = (op == XTG_RED_VARIANCE || op == XTG_RED_STDDEV) ? rd->ddof : 0;
    double div = n_out ? (double)((size - ddof) / n_out) : 0.0;
    /* write results (keep_dims: reduced dims are size 1 in out) */
    for (int64_t o = 0; o < n_out; ++o) {
        int64_t kidx[XTG_MAX_RANK], kshape[XTG_MAX_RANK];
        for (int i = 0; i < nk; ++i) kshape[i] = T.shape[kept[i]];
        unflat(o, nk, kshape, kidx);
        int64_t off = 0;
        int oi = 0, ki = 0;
        for (int d = 0; d < T.rank; ++d) {
            if (isred[d]) {
                if (rd->keep_dims) ++oi;
            } else {
                off += kidx[ki++] * out->strides[oi++];
            }
        }
        val r = res[o];
        if (rd->has_initial && op <= XTG_RED_AMIN) {
            val iv = is_float(r.t) ? mk_f(r.t, rd->initial.f) : mk_u(r.t, rd->initial.u);
            redctx c;
            c.op = op;
            c.acct = r.t;
            r = merge(&c, iv, r);
        }
        if (op == XTG_RED_MEAN) r = mk_f(XTG_FLOAT64, as_d(r) / div);
        if (op == XTG_RED_VARIANCE) r = mk_f(XTG_FLOAT64, as_d(r) / div);
        if (op == XTG_RED_STDDEV) r = mk_f(XTG_FLOAT64, sqrt(as_d(r) / div));
        if (op == XTG_RED_NORM_L2) r = mk_f(XTG_FLOAT64, sqrt(as_d(r)));
        store(out, off, r);
    }
    free(res);
    free(mean_at);
    return 0;
}

/* ---- arg reductions ----------------------------------------------------------------- */
int orc_argreduce(const xtg_expr* e, int op, int has_axis, int64_t axis, const xtg_array* out) {
    static otree T;
    int s = build(e, &T);
    if (s) return s;
    int R = T.rank;
    int ax = -1;
    if (has_axis && R > 1) {
        int64_t a = axis < 0 ? axis + R : axis;
        if (a < 0 || a >= R) return err(XTG_ERR_OUT_OF_RANGE, "axis");
        ax = (int)a;
    }
    int64_t total = 1;
    for (int d = 0; d < R; ++d) total *= T.shape[d];
    rowctx rc;
    int at = T.type[T.root];
    if (ax < 0) {
        /* flattened: std::max_element / std::min_element (first extreme) */
        int64_t best = 0, idx[XTG_MAX_RANK];
        unflat(0, R, T.shape, idx);
        val bv = eval(&T, T.root, idx, &rc);
        for (int64_t i = 1; i < total; ++i) {
            unflat(i, R, T.shape, idx);
            val v = eval(&T, T.root, idx, &rc);
            int better = op == XTG_ARGMAX ? cmp(XTG_OP_LT, at, bv, v) : cmp(XTG_OP_LT, at, v, bv);
            if (better) {
                bv = v;
                best = i;
            }
        }
        store(out, 0, mk_u(XTG_INT64, (uint64_t)best));
        return 0;
    }
    int64_t n = T.shape[ax];
    int64_t n_out = n ? total / n : 0;
    int kept[XTG_MAX_RANK], nk = 0;
    int64_t kshape[XTG_MAX_RANK];
    for (int d = 0; d < R; ++d)
        if (d != ax) {
            kshape[nk] = T.shape[d];
            kept[nk++] = d;
        }
#pragma omp parallel for schedule(static)
    for (int64_t o = 0; o < n_out; ++o) {
        int64_t kidx[XTG_MAX_RANK], idx[XTG_MAX_RANK] = {0};
        rowctx rc2;
        unflat(o, nk, kshape, kidx);
        for (int i = 0; i < nk; ++i) idx[kept[i]] = kidx[i];
        idx[ax] = 0;
        val bv = eval(&T, T.root, idx, &rc2);
        int64_t best = 0;
        for (int64_t j = 1; j < n; ++j) {
            idx[ax] = j;
            val v = eval(&T, T.root, idx, &rc2);
            if (op == XTG_ARGMAX ? cmp(XTG_OP_GT, at, v, bv) : cmp(XTG_OP_LT, at, v, bv)) {
                bv = v;
                best = j;
            }
        }
        int64_t off = 0;
        for (int i = 0; i < nk; ++i) off += kidx[i] * out->strides[i];
        store(out, off, mk_u(XTG_INT64, (uint64_t)best));
    }
    return 0;
}

/* ---- accumulators (cumsum / cumprod / nancumsum / nancumprod) ------------------------
 * xt::accumulate (include/xtensor/reducers/xaccumulator.hpp):
 *  - the result type is decltype(F(init_value_type, value_type)) (:206-214,
 *    :285-294): plus / multiplies of the template argument T (or the
 *    expression's value type) with the value type;
 *  - over an axis (:202-281): `result_type res = e` converts every element,
 *    then res[.., i, ..] = F(res[.., i-1, ..], res[.., i, ..]) for i >= 1 in
 *    that type (the nan variants first map res[.., 0, ..] through nan_init);
 *    an axis outside the expression is std::runtime_error (:217-220), the
 *    axis normalised by normalize_axis (include/xtensor/utils/xutils.hpp:353-357);
 *  - flattened (:283-310): a 1-D result of e.size() elements, result[0] =
 *    init(e_0), result[i] = F(result[i-1], e_i) in row-major order;
 *  - nan_plus / nan_multiplies skip NaN operands, nan_init maps NaN to 0 / 1
 *    (include/xtensor/core/xmath.hpp:2363-2391). */
static int val_isnan(val v) { return is_float(v.t) && v.f != v.f; }

int orc_accumulate_dtype(const xtg_expr* e, int op, int acc_dtype) {
    static otree T;
    int s = build(e, &T);
    if (s) return -s;
    (void)op;
    int vt = T.type[T.root];
    int it = acc_dtype >= 0 ? acc_dtype : vt;
    return orc_promote(it, vt);
}

static val acc_init(int op, val x) {
    if ((op == XTG_ACC_NANCUMSUM || op == XTG_ACC_NANCUMPROD) && val_isnan(x))
        return cvt(mk_u(XTG_INT64, op == XTG_ACC_NANCUMSUM ? 0 : 1), x.t);
    return x;
}
static val acc_step(int op, int rt, val acc, val x) {
    if ((op == XTG_ACC_NANCUMSUM || op == XTG_ACC_NANCUMPROD) && val_isnan(x)) return acc;
    return arith((op == XTG_ACC_CUMSUM || op == XTG_ACC_NANCUMSUM) ? XTG_OP_ADD : XTG_OP_MUL, rt, acc, x);
}

int orc_accumulate(const xtg_expr* e, int op, int has_axis, int64_t axis, int acc_dtype, const xtg_array* out) {
    static otree T;
    int s = build(e, &T);
    if (s) return s;
    int R = T.rank;
    int vt = T.type[T.root];
    int rt = orc_promote(acc_dtype >= 0 ? acc_dtype : vt, vt);
    if (out->dtype != rt) return err(XTG_ERR_INVALID, "destination dtype is not the accumulation type");
    int64_t total = 1;
    for (int d = 0; d < R; ++d) total *= T.shape[d];
    rowctx rc;
    if (!has_axis) {
        if (out->rank != 1 || out->shape[0] != total) return err(XTG_ERR_SHAPE, "flattened accumulation shape");
        val acc = mk_u(rt, 0);
        for (int64_t i = 0; i < total; ++i) {
            int64_t idx[XTG_MAX_RANK];
            unflat(i, R, T.shape, idx);
            val x = cvt(eval(&T, T.root, idx, &rc), rt);
            acc = i == 0 ? acc_init(op, x) : acc_step(op, rt, acc, x);
            store(out, i * out->strides[0], acc);
        }
        return 0;
    }
    int64_t a = axis < 0 ? axis + R : axis;
    if (a < 0 || a >= R) return err(XTG_ERR_AXIS, "Axis larger than expression dimension in accumulator.");
    if (out->rank != R) return err(XTG_ERR_SHAPE, "accumulation shape");
    for (int d = 0; d < R; ++d)
        if (out->shape[d] != T.shape[d]) return err(XTG_ERR_SHAPE, "accumulation shape");
    int ax = (int)a;
    int64_t n = T.shape[ax];
    int64_t n_out = n ? total / n : 0;
    int kept[XTG_MAX_RANK], nk = 0;
    int64_t kshape[XTG_MAX_RANK];
    for (int d = 0; d < R; ++d)
        if (d != ax) {
            kshape[nk] = T.shape[d];
            kept[nk++] = d;
        }
#pragma omp parallel for schedule(static)
    for (int64_t o = 0; o < n_out; ++o) {
        int64_t kidx[XTG_MAX_RANK], idx[XTG_MAX_RANK] = {0};
        rowctx rc2;
        unflat(o, nk, kshape, kidx);
        for (int i = 0; i < nk; ++i) idx[kept[i]] = kidx[i];
        val acc = mk_u(rt, 0);
        for (int64_t j = 0; j < n; ++j) {
            idx[ax] = j;
            val x = cvt(eval(&T, T.root, idx, &rc2), rt);
            acc = j == 0 ? acc_init(op, x) : acc_step(op, rt, acc, x);
            int64_t off = 0;
            for (int d = 0; d < R; ++d) off += idx[d] * out->strides[d];
            store(out, off, acc);
        }
    }
    return 0;
}
