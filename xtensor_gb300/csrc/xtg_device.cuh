// xtg_device.cuh — device side of the GB300 evaluator.
//
// This header is compiled two ways: by NVRTC (its text is embedded into
// libxtg.so; every expression tree is instantiated against it at first use,
// for sm_103a) and by nvcc (translation units that instantiate kernels ahead
// of time).  It uses no standard-library header so that NVRTC needs no
// include path.
//
// An expression tree is a C++ *type*: e.g. C0's `A*b + exp(-A*A)` becomes
//   Add<float, Mul<float, L<0,float>, L<1,float>>,
//              Exp<float, Neg<float, Mul<float, L<0,float>, L<0,float>>>>>
// — the lowered form of xtensor's xfunction<F, CT...>
// (include/xtensor/core/xfunction.hpp:203-375).  Each leaf is loaded once per
// element into registers (LeafSet), then the tree is evaluated as a pure
// function of those registers.  Broadcasting is stride-0 arithmetic in the
// per-leaf offset computation, which is what xtensor's steppers do with their
// `offset` / zero strides (include/xtensor/core/xiterator.hpp:488-497,
// include/xtensor/core/xstrides.hpp:570-581).
#pragma once

#ifndef XTG_DEVICE_CUH
#define XTG_DEVICE_CUH

#define XTG_DI __device__ __forceinline__

#include "xtg_params.h"

namespace xtg {


// ---------------------------------------------------------------------------
// bfloat16 storage type.  Conversions are written from the format definition:
// bf16 is the top 16 bits of an IEEE binary32; float -> bf16 rounds to
// nearest-even on the dropped 16 bits, NaN stays a quiet NaN.
struct bf16 {
    unsigned short bits;
    bf16() = default;  // trivial: bf16 lives in unions and shared memory
    XTG_DI bf16(float f) {
        u32 u = __float_as_uint(f);
        if ((u & 0x7fffffffu) > 0x7f800000u) {
            bits = (unsigned short)((u >> 16) | 0x40u);
        } else {
            u32 lsb = (u >> 16) & 1u;
            u += 0x7fffu + lsb;
            bits = (unsigned short)(u >> 16);
        }
    }
    XTG_DI bf16(double d) : bf16((float)d) {}
    XTG_DI bf16(int v) : bf16((float)v) {}
    XTG_DI bf16(long long v) : bf16((float)v) {}
    XTG_DI bf16(unsigned int v) : bf16((float)v) {}
    XTG_DI bf16(unsigned long long v) : bf16((float)v) {}
    XTG_DI operator float() const { return __uint_as_float(((u32)bits) << 16); }
};

// Programmatic dependent launch: the host may launch a kernel while the one
// before it in the stream still drains; every kernel waits here for its
// predecessors (their writes visible) before it touches global memory.
// Without the launch attribute this is a no-op.
XTG_DI void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Conversions: C++ static_cast semantics for arithmetic types, bf16 via float.
template <class To> struct Cvt {
    template <class From> static XTG_DI To go(From v) { return (To)v; }
    static XTG_DI To go(bf16 v) { return (To)(float)v; }
};
template <> struct Cvt<bf16> {
    template <class From> static XTG_DI bf16 go(From v) { return bf16((float)v); }
    static XTG_DI bf16 go(double v) { return bf16((float)v); }
    static XTG_DI bf16 go(bf16 v) { return v; }
};
template <> struct Cvt<bool> {
    template <class From> static XTG_DI bool go(From v) { return v != From(0); }
    static XTG_DI bool go(bf16 v) { return (float)v != 0.f; }
    static XTG_DI bool go(bool v) { return v; }
};
template <class To, class From> XTG_DI To cvt(From v) { return Cvt<To>::go(v); }

// Numeric limits needed for reducer initial values (amax/amin use lowest()/max()).
template <class T> struct Lim;
template <> struct Lim<bool> { static XTG_DI bool lowest() { return false; } static XTG_DI bool maxv() { return true; } };
template <> struct Lim<signed char> { static XTG_DI signed char lowest() { return -128; } static XTG_DI signed char maxv() { return 127; } };
template <> struct Lim<unsigned char> { static XTG_DI unsigned char lowest() { return 0; } static XTG_DI unsigned char maxv() { return 255; } };
template <> struct Lim<short> { static XTG_DI short lowest() { return -32768; } static XTG_DI short maxv() { return 32767; } };
template <> struct Lim<unsigned short> { static XTG_DI unsigned short lowest() { return 0; } static XTG_DI unsigned short maxv() { return 65535; } };
template <> struct Lim<int> { static XTG_DI int lowest() { return (-2147483647 - 1); } static XTG_DI int maxv() { return 2147483647; } };
template <> struct Lim<unsigned int> { static XTG_DI unsigned int lowest() { return 0u; } static XTG_DI unsigned int maxv() { return 4294967295u; } };
template <> struct Lim<long long> { static XTG_DI long long lowest() { return (-9223372036854775807LL - 1); } static XTG_DI long long maxv() { return 9223372036854775807LL; } };
template <> struct Lim<unsigned long long> { static XTG_DI unsigned long long lowest() { return 0ull; } static XTG_DI unsigned long long maxv() { return 18446744073709551615ull; } };
template <> struct Lim<float> { static XTG_DI float lowest() { return -3.40282346638528859812e+38f; } static XTG_DI float maxv() { return 3.40282346638528859812e+38f; } };
template <> struct Lim<double> { static XTG_DI double lowest() { return -1.7976931348623157e+308; } static XTG_DI double maxv() { return 1.7976931348623157e+308; } };

template <class T> struct IsFloat { enum { value = 0 }; };
template <> struct IsFloat<float> { enum { value = 1 }; };
template <> struct IsFloat<double> { enum { value = 1 }; };
template <> struct IsFloat<bf16> { enum { value = 1 }; };

// ---------------------------------------------------------------------------
// Fast unsigned 32-bit division by a run-time invariant divisor, by the
// round-up multiply-and-shift method of Granlund & Montgomery (PLDI 1994):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (mulhi(m, n) + n) >> l, exact for all n < 2^32.
XTG_DI u32 fdiv(u32 n, const FastDiv& f) {
    u32 t = __umulhi(f.m, n);
    return (u32)(((u64)t + n) >> f.l);
}

// ---------------------------------------------------------------------------
// Kernel parameter blocks.  Strides/shapes are in elements; offsets 64-bit.
template <class T> XTG_DI T scalar_as(const Scalars& s, int k);
template <> XTG_DI float scalar_as<float>(const Scalars& s, int k) { return (float)__longlong_as_double((i64)s.v[k]); }
template <> XTG_DI double scalar_as<double>(const Scalars& s, int k) { return __longlong_as_double((i64)s.v[k]); }
template <> XTG_DI bf16 scalar_as<bf16>(const Scalars& s, int k) { return bf16((float)__longlong_as_double((i64)s.v[k])); }
template <> XTG_DI bool scalar_as<bool>(const Scalars& s, int k) { return s.v[k] != 0; }
template <> XTG_DI signed char scalar_as<signed char>(const Scalars& s, int k) { return (signed char)(i64)s.v[k]; }
template <> XTG_DI unsigned char scalar_as<unsigned char>(const Scalars& s, int k) { return (unsigned char)s.v[k]; }
template <> XTG_DI short scalar_as<short>(const Scalars& s, int k) { return (short)(i64)s.v[k]; }
template <> XTG_DI unsigned short scalar_as<unsigned short>(const Scalars& s, int k) { return (unsigned short)s.v[k]; }
template <> XTG_DI int scalar_as<int>(const Scalars& s, int k) { return (int)(i64)s.v[k]; }
template <> XTG_DI unsigned int scalar_as<unsigned int>(const Scalars& s, int k) { return (unsigned int)s.v[k]; }
template <> XTG_DI long long scalar_as<long long>(const Scalars& s, int k) { return (i64)s.v[k]; }
template <> XTG_DI unsigned long long scalar_as<unsigned long long>(const Scalars& s, int k) { return s.v[k]; }

// Decode a flat vector index into a multi-index (innermost in elements).
template <int R, int VEC, bool BIG>
XTG_DI void decode(const Space& sp, i64 q, i64 (&idx)[R]) {
    if (BIG) {
#pragma unroll
        for (int d = R - 1; d >= 0; --d) {
            i64 n = sp.shape[d];
            i64 qq = q / n;
            idx[d] = q - qq * n;
            q = qq;
        }
    } else {
        u32 qu = (u32)q;
#pragma unroll
        for (int d = R - 1; d >= 0; --d) {
            if (d == 0) {
                idx[0] = qu;
            } else {
                u32 qq = fdiv(qu, sp.fd[d]);
                idx[d] = qu - qq * sp.fd[d].d;
                qu = qq;
            }
        }
    }
    idx[R - 1] *= VEC;
}

template <int R>
XTG_DI i64 dot_idx(const i64 (&idx)[R], const i64* st) {
    i64 o = 0;
#pragma unroll
    for (int d = 0; d < R; ++d) o += idx[d] * st[d];
    return o;
}

// ---------------------------------------------------------------------------
// Vector memory access.  VEC elements of T at p (p aligned to VEC*sizeof(T)
// when KIND == CONTIG, which the host checks before choosing VEC > 1).
enum { K_CONTIG = 0, K_BCAST = 1, K_STRIDED = 2 };

template <int BYTES> struct VecT;
template <> struct VecT<16> { typedef uint4 t; };
template <> struct VecT<8> { typedef uint2 t; };
template <> struct VecT<4> { typedef unsigned int t; };
template <> struct VecT<2> { typedef unsigned short t; };
template <> struct VecT<1> { typedef unsigned char t; };

template <class T, int VEC>
XTG_DI void ld_contig(T (&dst)[VEC], const T* p) {
    const int B = (int)sizeof(T) * VEC;
    if (B == 16 || B == 8 || B == 4 || B == 2) {
        typedef typename VecT<(B > 16 ? 16 : B)>::t V;
        union { V v; T e[VEC]; } u;
        u.v = __ldg(reinterpret_cast<const V*>(p));
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = u.e[j];
    } else if (B == 32) {
        union { uint4 v[2]; T e[VEC]; } u;
        u.v[0] = __ldg(reinterpret_cast<const uint4*>(p));
        u.v[1] = __ldg(reinterpret_cast<const uint4*>(p) + 1);
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = u.e[j];
    } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = p[j];
    }
}
// bool / bf16 / 1-byte types: __ldg has no overload for them, route via bytes.
template <class T> XTG_DI T ld1(const T* p) { return *p; }
template <> XTG_DI float ld1<float>(const float* p) { return __ldg(p); }
template <> XTG_DI double ld1<double>(const double* p) { return __ldg(p); }
template <> XTG_DI int ld1<int>(const int* p) { return __ldg(p); }
template <> XTG_DI long long ld1<long long>(const long long* p) { return __ldg(p); }

template <class T, int KIND, int VEC>
XTG_DI void ld_leaf(T (&dst)[VEC], const T* base, i64 off, i64 inner_stride) {
    if (KIND == K_CONTIG) {
        ld_contig<T, VEC>(dst, base + off);
    } else if (KIND == K_BCAST) {
        T v = ld1<T>(base + off);
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = v;
    } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = ld1<T>(base + off + (i64)j * inner_stride);
    }
}

template <class T, int KIND, int VEC>
XTG_DI void st_out(T* base, i64 off, i64 inner_stride, const T (&v)[VEC]) {
    const int B = (int)sizeof(T) * VEC;
    if (KIND == K_CONTIG && (B == 16 || B == 8 || B == 4 || B == 2)) {
        typedef typename VecT<(B > 16 ? 16 : B)>::t V;
        union { V v; T e[VEC]; } u;
#pragma unroll
        for (int j = 0; j < VEC; ++j) u.e[j] = v[j];
        *reinterpret_cast<V*>(base + off) = u.v;
    } else if (KIND == K_CONTIG && B == 32) {
        union { uint4 v[2]; T e[VEC]; } u;
#pragma unroll
        for (int j = 0; j < VEC; ++j) u.e[j] = v[j];
        reinterpret_cast<uint4*>(base + off)[0] = u.v[0];
        reinterpret_cast<uint4*>(base + off)[1] = u.v[1];
    } else if (KIND == K_CONTIG) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) base[off + j] = v[j];
    } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) base[off + (i64)j * inner_stride] = v[j];
    }
}

// ---------------------------------------------------------------------------
// Leaf sets: a compile-time list of (type, access kind) and the register
// storage for VEC values of each.
template <class T, int KIND> struct LeafSpec {
    typedef T type;
    enum { kind = KIND };
};

template <int VEC, class... S> struct Regs;
template <int VEC> struct Regs<VEC> {};
template <int VEC, class S0, class... S> struct Regs<VEC, S0, S...> {
    typedef typename S0::type elem0;
    typename S0::type v[VEC];
    Regs<VEC, S...> rest;
};
template <int I> struct RegAt {
    template <class R> static XTG_DI auto& get(R& r) { return RegAt<I - 1>::get(r.rest); }
    template <class R> static XTG_DI const auto& cget(const R& r) { return RegAt<I - 1>::cget(r.rest); }
};
template <> struct RegAt<0> {
    template <class R> static XTG_DI auto& get(R& r) { return r.v; }
    template <class R> static XTG_DI const auto& cget(const R& r) { return r.v; }
};

template <class... S> struct LeafSet {
    enum { N = sizeof...(S) };
    template <int VEC> struct R { typedef Regs<VEC, S...> type; };
};

// Load all leaves for one vector position; offsets from a multi-index.
template <int I, int VEC, int R, class... S> struct LoadAll;
template <int I, int VEC, int R> struct LoadAll<I, VEC, R> {
    template <class RG> static XTG_DI void run(RG&, const void* const*, const i64 (*)[XTG_KMAX_RANK], const i64 (&)[R]) {}
};
template <int I, int VEC, int R, class S0, class... S> struct LoadAll<I, VEC, R, S0, S...> {
    template <class RG>
    static XTG_DI void run(RG& rg, const void* const* ptr, const i64 (*st)[XTG_KMAX_RANK], const i64 (&idx)[R]) {
        typedef typename S0::type T;
        i64 off = dot_idx<R>(idx, st[I]);
        ld_leaf<T, S0::kind, VEC>(rg.v, reinterpret_cast<const T*>(ptr[I]), off, st[I][R - 1]);
        LoadAll<I + 1, VEC, R, S...>::run(rg.rest, ptr, st, idx);
    }
};
template <class LS> struct LoadLeaves;
template <class... S> struct LoadLeaves<LeafSet<S...>> {
    template <int VEC, int R, class RG>
    static XTG_DI void run(RG& rg, const void* const* ptr, const i64 (*st)[XTG_KMAX_RANK], const i64 (&idx)[R]) {
        LoadAll<0, VEC, R, S...>::run(rg, ptr, st, idx);
    }
};

// ---------------------------------------------------------------------------
// Evaluation context: scalar immediates plus row statistics (for the fused
// row kernels).  Nodes evaluate at vector lane j.
template <int NSTAT> struct Ctx {
    Scalars scal;  // by value: immediates live in registers, conversions hoist
    double stat[NSTAT > 0 ? NSTAT : 1];   // row statistics (FP64 consumers)
    float statf[NSTAT > 0 ? NSTAT : 1];   // the same, rounded once (FP32 consumers)
    unsigned fixmask;                     // statistics already produced for this row (bit K)
};

// Leaves / scalars / row statistics as tree terminals.
template <int I, class T> struct L {
    typedef T type;
    template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C&) { return RegAt<I>::cget(r)[j]; }
};
template <int K, class T> struct S {
    typedef T type;
    template <class RG, class C> static XTG_DI T ev(const RG&, int, const C& c) { return scalar_as<T>(c.scal, K); }
};
// A row statistic produced by a fused row reducer (index K of Ctx::stat).
template <class T> struct StatGet {
    template <class C> static XTG_DI T get(const C& c, int k) { return (T)c.stat[k]; }
    template <class C> static XTG_DI void put(C& c, int k, T v) {
        c.stat[k] = (double)v;
        c.statf[k] = (float)v;
    }
};
template <> struct StatGet<float> {
    template <class C> static XTG_DI float get(const C& c, int k) { return c.statf[k]; }
    template <class C> static XTG_DI void put(C& c, int k, float v) {
        c.statf[k] = v;
        c.stat[k] = (double)v;
    }
};
// Row-invariant subtrees evaluated once per row before the output pass: the
// reciprocal nodes (MulRecip, FmaRecipSub) store theirs in statistic slots
// after the real statistics.  Prep walks the tree; nodes without work recurse.
template <class N> struct Prep {
    template <class RG, class C> static XTG_DI void run(const RG&, C&) {}
};
template <template <class...> class N, class... X> struct Prep<N<X...>> {
    template <class RG, class C> static XTG_DI void run(const RG& r, C& c) { (Prep<X>::run(r, c), ...); }
};
template <int K, class T> struct Stat {
    typedef T type;
    template <class RG, class C> static XTG_DI T ev(const RG&, int, const C& c) { return StatGet<T>::get(c, K); }
};

// Unary functors (include/xtensor/core/xoperation.hpp:104-125,
// include/xtensor/core/xmath.hpp:295-341, 1101-1108).
#define XTG_UNARY(NAME, EXPR)                                                              \
    template <class T, class A> struct NAME {                                              \
        typedef T type;                                                                    \
        template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C& c) {   \
            typedef typename A::type TA;                                                   \
            T a = cvt<T>(A::ev(r, j, c));                                                  \
            (void)sizeof(TA);                                                              \
            return EXPR;                                                                   \
        }                                                                                  \
    };
XTG_UNARY(Neg, (T)(-a))
XTG_UNARY(Pos, (T)(+a))
XTG_UNARY(Square, (T)(a * a))
XTG_UNARY(LogicalNot, (T)(!a))
XTG_UNARY(BitNot, (T)(~a))
XTG_UNARY(Cast, a)
#undef XTG_UNARY

// Math functions: float overloads call the single-precision CUDA functions,
// double overloads the double ones (std::exp(float) vs std::exp(double)).
XTG_DI float m_exp(float x) { return expf(x); }
XTG_DI double m_exp(double x) { return exp(x); }
XTG_DI float m_log(float x) { return logf(x); }
XTG_DI double m_log(double x) { return log(x); }
XTG_DI float m_sqrt(float x) { return sqrtf(x); }
XTG_DI double m_sqrt(double x) { return sqrt(x); }
XTG_DI float m_sin(float x) { return sinf(x); }
XTG_DI double m_sin(double x) { return sin(x); }
XTG_DI float m_cos(float x) { return cosf(x); }
XTG_DI double m_cos(double x) { return cos(x); }
XTG_DI float m_tanh(float x) { return tanhf(x); }
XTG_DI double m_tanh(double x) { return tanh(x); }
XTG_DI float m_pow(float x, float y) { return powf(x, y); }
XTG_DI double m_pow(double x, double y) { return pow(x, y); }
template <class T> XTG_DI T m_abs(T x) { return x < T(0) ? T(-x) : x; }
XTG_DI float m_abs(float x) { return fabsf(x); }
XTG_DI double m_abs(double x) { return fabs(x); }

#define XTG_MATH1(NAME, FN)                                                               \
    template <class T, class A> struct NAME {                                             \
        typedef T type;                                                                   \
        template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C& c) {  \
            return FN(cvt<T>(A::ev(r, j, c)));                                            \
        }                                                                                 \
    };
XTG_MATH1(Exp, m_exp)
XTG_MATH1(Log, m_log)
XTG_MATH1(Sqrt, m_sqrt)
XTG_MATH1(Abs, m_abs)
XTG_MATH1(Sin, m_sin)
XTG_MATH1(Cos, m_cos)
XTG_MATH1(Tanh, m_tanh)
#undef XTG_MATH1

// Binary arithmetic: operands converted to the node type T (the C++ common
// type the host computed), then the operator applied.
#define XTG_BINARY(NAME, EXPR)                                                            \
    template <class T, class A, class B> struct NAME {                                    \
        typedef T type;                                                                   \
        template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C& c) {  \
            T a = cvt<T>(A::ev(r, j, c));                                                 \
            T b = cvt<T>(B::ev(r, j, c));                                                 \
            return EXPR;                                                                  \
        }                                                                                 \
    };
XTG_BINARY(Add, (T)(a + b))
XTG_BINARY(Sub, (T)(a - b))
XTG_BINARY(Mul, (T)(a * b))
XTG_BINARY(Div, (T)(a / b))
XTG_BINARY(Mod, (T)(a % b))
XTG_BINARY(BitAnd, (T)(a & b))
XTG_BINARY(BitOr, (T)(a | b))
XTG_BINARY(BitXor, (T)(a ^ b))
XTG_BINARY(Pow, m_pow(a, b))
// maximum/minimum keep the reference's select order: select(t1 > t2, t1, t2)
// (include/xtensor/core/xmath.hpp:589-602).
XTG_BINARY(Maximum, (a > b ? a : b))
XTG_BINARY(Minimum, (a < b ? a : b))
#undef XTG_BINARY

// Comparisons and logical ops: computed in the common type CT, result bool.
#define XTG_CMP(NAME, OP)                                                                 \
    template <class CT, class A, class B> struct NAME {                                   \
        typedef bool type;                                                                \
        template <class RG, class C> static XTG_DI bool ev(const RG& r, int j, const C& c) { \
            CT a = cvt<CT>(A::ev(r, j, c));                                               \
            CT b = cvt<CT>(B::ev(r, j, c));                                               \
            return a OP b;                                                                \
        }                                                                                 \
    };
XTG_CMP(Lt, <)
XTG_CMP(Le, <=)
XTG_CMP(Gt, >)
XTG_CMP(Ge, >=)
XTG_CMP(Eq, ==)
XTG_CMP(Ne, !=)
XTG_CMP(LogicalAnd, &&)
XTG_CMP(LogicalOr, ||)
#undef XTG_CMP

template <class T, class Cd, class A, class B> struct Where {
    typedef T type;
    template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C& c) {
        return cvt<bool>(Cd::ev(r, j, c)) ? cvt<T>(A::ev(r, j, c)) : cvt<T>(B::ev(r, j, c));
    }
};

// ---------------------------------------------------------------------------
// K1: fused elementwise assignment  out[i] = Tree(leaves at i)
// Replaces linear_assigner / strided_loop_assigner / stepper_assigner
// (include/xtensor/core/xassign.hpp:644-695, 701-849, 855-1358) for any
// destination and leaf strides.  Grid-stride over vectors of VEC elements;
// each thread keeps U independent vectors in flight (U * leaves * 16 B of
// loads outstanding) so that HBM latency is hidden with few CTAs per SM.
template <class Tree, class LS, class OutT, int OUTKIND, int VEC, int R, int U, bool BIG>
__global__ void __launch_bounds__(256) k_assign(const AssignParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    Ctx<0> c;
    c.scal = p.scal;
    const i64 step = (i64)gridDim.x * blockDim.x * U;
    for (i64 base = (i64)blockIdx.x * blockDim.x * U + threadIdx.x; base < p.sp.nvec; base += step) {
        RG rg[U];
        i64 ooff[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            i64 q = base + (i64)u * blockDim.x;
            if (q < p.sp.nvec) {
                i64 idx[R];
                decode<R, VEC, BIG>(p.sp, q, idx);
                LoadLeaves<LS>::template run<VEC, R>(rg[u], p.leaf, p.leaf_strides, idx);
                ooff[u] = dot_idx<R>(idx, p.out_strides);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            i64 q = base + (i64)u * blockDim.x;
            if (q < p.sp.nvec) {
                OutT v[VEC];
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[j] = cvt<OutT>(Tree::ev(rg[u], j, c));
                st_out<OutT, OUTKIND, VEC>(reinterpret_cast<OutT*>(p.out), ooff[u], p.out_strides[R - 1], v);
            }
        }
    }
}


// ---------------------------------------------------------------------------
// K12: assignment over a chunk grid (xchunked_semantic::assign_xexpression,
// include/xtensor/chunk/xchunked_assign.hpp:200-219): every chunk's region of
// the expression into the chunk, for all chunks in one launch.  The chunks
// come in classes of equal valid extents; the launch walks the classes in
// turn, and inside a class work item q = (chunk, vector of the chunk's valid
// region), so no thread lands in the padding of an edge chunk.  The host
// picks VEC so that it divides every class's innermost extent.  PAD (more
// classes than the parameter block holds): one class of padded chunks, the
// entries' extents bound the elements.
template <class Tree, class LS, class OutT, int OUTKIND, int VEC, int R, int U, bool BIG, bool PAD = false>
__global__ void __launch_bounds__(256) k_assign_chunks(const ChunkParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    Ctx<0> c;
    c.scal = p.scal;
    const i64 step = (i64)gridDim.x * blockDim.x * U;
    for (int k = 0; k < p.n_cls; ++k) {
        const ChunkClass& K = p.cls[k];
        const i64 nv = K.sp.nvec;
        const i64 total = K.count * nv;
        for (i64 base = (i64)blockIdx.x * blockDim.x * U + threadIdx.x; base < total; base += step) {
            RG rg[U];
            i64 ooff[U];
            void* optr[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const i64 q = base + (i64)u * blockDim.x;
                ok[u] = false;
                if (q < total) {
                    i64 ch, loc;
                    if (BIG) {
                        ch = q / nv;
                        loc = q - ch * nv;
                    } else {
                        const u32 qq = fdiv((u32)q, K.fdn);
                        ch = qq;
                        loc = (u32)q - qq * K.fdn.d;
                    }
                    i64 idx[R];
                    decode<R, VEC, BIG>(K.sp, loc, idx);
                    const ChunkEntry& ent = p.tab[K.first + ch];
                    bool in = true;
                    if (PAD) {
#pragma unroll
                        for (int d = 0; d < R; ++d) in = in && idx[d] < ent.ext[d];
                    }
                    if (in) {
                        ok[u] = true;
                        LoadLeaves<LS>::template run<VEC, R>(rg[u], ent.leaf, p.leaf_strides, idx);
                        ooff[u] = dot_idx<R>(idx, p.out_strides);
                        optr[u] = ent.out;
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (ok[u]) {
                    OutT v[VEC];
#pragma unroll
                    for (int j = 0; j < VEC; ++j) v[j] = cvt<OutT>(Tree::ev(rg[u], j, c));
                    st_out<OutT, OUTKIND, VEC>(reinterpret_cast<OutT*>(optr[u]), ooff[u], p.out_strides[R - 1], v);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Generic warp shuffle of a POD accumulator (word by word).
template <class A> XTG_DI A shfl_xor_pod(const A& a, int m) {
    union U { A a; u32 w[(sizeof(A) + 3) / 4]; };
    U in, out;
    in.a = a;
#pragma unroll
    for (int i = 0; i < (int)((sizeof(A) + 3) / 4); ++i) out.w[i] = __shfl_xor_sync(0xffffffffu, in.w[i], m);
    return out.a;
}

template <class A> XTG_DI A shfl_up_pod(const A& a, int d) {
    union U { A a; u32 w[(sizeof(A) + 3) / 4]; };
    U in, out;
    in.a = a;
#pragma unroll
    for (int i = 0; i < (int)((sizeof(A) + 3) / 4); ++i) out.w[i] = __shfl_up_sync(0xffffffffu, in.w[i], d);
    return out.a;
}

template <class A> XTG_DI A shfl_idx_pod(const A& a, int src) {
    union U { A a; u32 w[(sizeof(A) + 3) / 4]; };
    U in, out;
    in.a = a;
#pragma unroll
    for (int i = 0; i < (int)((sizeof(A) + 3) / 4); ++i) out.w[i] = __shfl_sync(0xffffffffu, in.w[i], src);
    return out.a;
}

// Deterministic group reduction: warp butterfly, then warp 0 folds the
// per-warp results in warp order.  Result valid in thread 0 of the group
// (GROUP == 32: lane 0 of the warp; GROUP == block: thread 0).
template <int GROUP, class A> XTG_DI A group_reduce(A a, A* smem) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        A o = shfl_xor_pod(a, m);
        a.merge(o);
    }
    if (GROUP <= 32) return a;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) smem[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        A r = smem[0];
        for (int w = 1; w < nw; ++w) r.merge(smem[w]);
        a = r;
    }
    return a;
}

// Knuth's TwoSum: s = fl(a + b), e = (a + b) - s exactly.
XTG_DI void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Packed float32 pairs: one instruction advances two independent FP32
// operations (sm_100+ FADD2 / FMUL2 / FFMA2).  a - b is fma(b, -1, a): the
// exact difference rounded once, the same result as the subtraction (round
// to nearest is symmetric, so fl(b - a) = -fl(a - b) as well).
XTG_DI float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
XTG_DI float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
XTG_DI float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
XTG_DI float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// TwoSum on both lanes: s + e == a + b exactly, lane by lane.
XTG_DI void two_sum2(float2 a, float2 b, float2& s, float2& e) {
    s = p_add(a, b);
    const float2 bb = p_sub(s, a);
    e = p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb));
}

// Pairwise sums of 2N float32 values held as N pairs, with packed
// instructions: lane x sums the even values, lane y the odd ones, and x + y
// closes the tree — depth log2(2N), so the rounding error of the whole sum
// is at most ceil(log2 2N) u sum |f| (u = 2^-24).  Squares: pairs as
// fma(a, a, b * b), then pairwise.
template <int N> struct Pw2 {
    static XTG_DI float2 sum(const float2* f) { return p_add(Pw2<N / 2>::sum(f), Pw2<N - N / 2>::sum(f + N / 2)); }
    static XTG_DI float2 sq(const float2* f) { return p_add(Pw2<N / 2>::sq(f), Pw2<N - N / 2>::sq(f + N / 2)); }
};
template <> struct Pw2<1> {
    static XTG_DI float2 sum(const float2* f) { return f[0]; }
    static XTG_DI float2 sq(const float2* f) { return p_mul(f[0], f[0]); }
};
template <> struct Pw2<2> {
    static XTG_DI float2 sum(const float2* f) { return p_add(f[0], f[1]); }
    static XTG_DI float2 sq(const float2* f) { return p_fma(f[0], f[0], p_mul(f[1], f[1])); }
};

// ---------------------------------------------------------------------------
// Reduction accumulators.  Each is POD: init(p), add(x, pos), merge(other),
// and result<Out>(p).  `pos` is the element's row-major position inside the
// reduced index space; only the selection reducers use it.

// Plain accumulation in the accumulator type A (integers: exact modulo 2^n,
// so any order gives the reference's result bit for bit; float64: FP64).
// OP 0 = plus, 1 = multiplies (XTENSOR_REDUCER_FUNCTION sum / prod,
// include/xtensor/core/xmath.hpp:1803,1823).
template <class A, int OP> struct AccPlain {
    A s;
    template <class P> XTG_DI void init(const P& p);
    template <class X> XTG_DI void add(X x, i64) {
        if (OP == 0) s = (A)(s + cvt<A>(x)); else s = (A)(s * cvt<A>(x));
    }
    XTG_DI void merge(const AccPlain& o) {
        if (OP == 0) s = (A)(s + o.s); else s = (A)(s * o.s);
    }
    XTG_DI double dval() const { return (double)s; }
};

// float32 compensated sum: (hi, lo) double-float accumulation with TwoSum at
// every add and every merge, so the compensation survives the warp, block and
// grid combines.
struct AccSumC {
    float hi, lo;
    template <class P> XTG_DI void init(const P& p);
    template <class X> XTG_DI void add(X x, i64) {
        float v = cvt<float>(x), s, e;
        two_sum(hi, v, s, e);
        hi = s;
        lo += e;
    }
    XTG_DI void addf(float v) {
        float s, e;
        two_sum(hi, v, s, e);
        hi = s;
        lo += e;
    }
    XTG_DI void merge(const AccSumC& o) {
        float s, e;
        two_sum(hi, o.hi, s, e);
        hi = s;
        lo = (lo + o.lo) + e;
    }
    XTG_DI double dval() const { return (double)hi + (double)lo; }
};

template <class T> struct Cmp {
    static XTG_DI bool gt(T a, T b) { return a > b; }
    static XTG_DI bool lt(T a, T b) { return a < b; }
};

// Selection reducers amax / amin: the reference folds f(acc, x) =
// acc > x ? acc : x (include/xtensor/core/xmath.hpp:589-602, 777-811) from
// lowest()/max(), so among equal values the LAST one visited wins (this is
// visible for +0/-0).  The position makes that rule order-independent.
template <class A, int MAXOP> struct AccSel {
    A v;
    i64 pos;
    template <class P> XTG_DI void init(const P& p);
    XTG_DI void start(A v0) {
        v = v0;
        pos = -1;
    }
    XTG_DI A value() const { return v; }
    template <class X> XTG_DI void add(X x, i64 ps) {
        A a = cvt<A>(x);
        bool keep = MAXOP ? Cmp<A>::gt(v, a) : Cmp<A>::lt(v, a);
        if (!keep) { v = a; pos = ps; }
    }
    XTG_DI void merge(const AccSel& o) {
        bool take;
        if (MAXOP) take = Cmp<A>::gt(o.v, v) || (!Cmp<A>::gt(v, o.v) && o.pos > pos);
        else take = Cmp<A>::lt(o.v, v) || (!Cmp<A>::lt(v, o.v) && o.pos > pos);
        if (take) { v = o.v; pos = o.pos; }
    }
    XTG_DI double dval() const { return (double)v; }
};

// float64 order on the integer pipes (GB300 issues FP64 compares at its
// reduced FP64 rate).  key64 maps the bits of every non-NaN double to a signed
// integer in the same order (-0 lands just below +0); it is its own inverse.
// "Special" values — zeros, subnormals below 2^-1042, infinities and NaNs
// (high word magnitude 0 or >= 0x7ff00000) — take an exact IEEE path out of
// line (-0 == +0, NaN rules); between any other value and the running best,
// whatever that is, the key order is the IEEE order.
XTG_DI i64 key64(i64 b) { return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }
XTG_DI double unkey64(i64 k) { return __longlong_as_double(key64(k)); }
XTG_DI bool f64_special(i64 b) { return (unsigned)(((int)(b >> 32) & 0x7fffffff) - 1) >= 0x7fefffffu; }
XTG_DI bool f64_isnan_bits(i64 b) { return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
#define XTG_KEY_MIN ((i64)0x8000000000000000ULL)  // unkey64 of either end is a NaN
#define XTG_KEY_MAX ((i64)0x7fffffffffffffffLL)
struct KeyPos {
    i64 k, p;
};
// amax/amin update by a special value: the plain fold `keep = v > a`; a NaN
// best is stored as the end key that lets the next element in (the fold
// replaces a NaN accumulator by whatever follows).
template <int MAXOP> __device__ __noinline__ KeyPos sel_special(i64 kv, i64 pos, double a, i64 ps) {
    const double v = unkey64(kv);
    const bool keep = MAXOP ? (v > a) : (v < a);
    KeyPos r;
    r.k = kv;
    r.p = pos;
    if (!keep) {
        const i64 b = __double_as_longlong(a);
        r.k = f64_isnan_bits(b) ? (MAXOP ? XTG_KEY_MIN : XTG_KEY_MAX) : key64(b);
        r.p = ps;
    }
    return r;
}
template <int MAXOP> struct AccSel<double, MAXOP> {
    i64 kv;  // key64 of the best value
    i64 pos;
    template <class P> XTG_DI void init(const P& p) { start(p.init_f); }
    XTG_DI void start(double v0) {
        const i64 b = __double_as_longlong(v0);
        kv = f64_isnan_bits(b) ? (MAXOP ? XTG_KEY_MIN : XTG_KEY_MAX) : key64(b);
        pos = -1;
    }
    XTG_DI double value() const { return unkey64(kv); }
    template <class X> XTG_DI void add(X x, i64 ps) {
        const i64 b = __double_as_longlong(cvt<double>(x));
        if (f64_special(b)) {
            const KeyPos r = sel_special<MAXOP>(kv, pos, __longlong_as_double(b), ps);
            kv = r.k;
            pos = r.p;
            return;
        }
        const i64 ka = key64(b);
        if (MAXOP ? (ka >= kv) : (ka <= kv)) {  // equal keys = equal values: the later one wins
            kv = ka;
            pos = ps;
        }
    }
    XTG_DI void merge(const AccSel& o) {
        const double v = value(), ov = o.value();
        bool take;
        if (MAXOP) take = (ov > v) || (!(v > ov) && o.pos > pos);
        else take = (ov < v) || (!(v < ov) && o.pos > pos);
        if (take) {
            kv = o.kv;
            pos = o.pos;
        }
    }
    XTG_DI double dval() const { return value(); }
};

// Position-free selection for the row kernel's first pass.  Positions only
// decide between values that compare equal with different bits (+0 / -0) and
// around NaNs; a pass that met neither keeps the plain best value (equal
// values then have equal bits, so any merge order gives the same result).
// A pass that met a NaN, or ends on a zero (float) / a key64 special value
// (double), asks for the exact pass with positions.
template <class A, int MAXOP> struct AccSelFast {
    A v;
    bool odd;
    template <class P> XTG_DI void init(const P& p) {
        v = IsFloat<A>::value ? (A)p.init_f : (A)p.init_i;
        odd = false;
    }
    template <class X> XTG_DI void add(X x, i64) {
        const A a = cvt<A>(x);
        if (IsFloat<A>::value) odd |= !(a == a);
        const bool keep = MAXOP ? Cmp<A>::gt(v, a) : Cmp<A>::lt(v, a);
        if (!keep) v = a;
    }
    XTG_DI bool exact() const { return odd || (IsFloat<A>::value && v == A(0)); }
    XTG_DI void to(AccSel<A, MAXOP>& s) const {
        s.v = v;
        s.pos = -1;
    }
};
// float: one NaN-propagating max / min per element (PTX max.NaN / min.NaN):
// the running value turns NaN at the first NaN and stays NaN, which asks for
// the exact pass; otherwise it is the plain fold's value.
XTG_DI float fsel_nan(float a, float b, int maxop) {
    float r;
    if (maxop) asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    else asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
template <int MAXOP> struct AccSelFast<float, MAXOP> {
    float v;
    template <class P> XTG_DI void init(const P& p) { v = (float)p.init_f; }
    template <class X> XTG_DI void add(X x, i64) { v = fsel_nan(v, cvt<float>(x), MAXOP); }
    XTG_DI bool exact() const { return !(v == v) || v == 0.f; }
    XTG_DI void to(AccSel<float, MAXOP>& s) const {
        s.v = v;
        s.pos = -1;
    }
};
// double: the key order is the IEEE order except for NaNs and for -0 / +0,
// so the pass keeps the largest high word magnitude (an infinity or NaN
// anywhere asks for the exact pass) and asks for it too when the best key is
// a zero's (0: +0, -1: -0), where the fold's last-visited rule decides.
template <int MAXOP> struct AccSelFast<double, MAXOP> {
    i64 kv;
    unsigned mh;  // largest (high word & 0x7fffffff) seen
    bool odd;
    template <class P> XTG_DI void init(const P& p) {
        AccSel<double, MAXOP> s;
        s.start(p.init_f);
        kv = s.kv;
        mh = 0;
        odd = f64_special(__double_as_longlong(p.init_f));
    }
    template <class X> XTG_DI void add(X x, i64) {
        const i64 b = __double_as_longlong(cvt<double>(x));
        const unsigned h = (unsigned)(b >> 32) & 0x7fffffffu;
        mh = mh > h ? mh : h;
        const i64 ka = key64(b);
        if (MAXOP ? (ka >= kv) : (ka <= kv)) kv = ka;
    }
    XTG_DI bool exact() const { return odd || mh >= 0x7ff00000u || kv == 0 || kv == -1; }
    XTG_DI void to(AccSel<double, MAXOP>& s) const {
        s.kv = kv;
        s.pos = -1;
    }
};
template <class A> struct FastSel { enum { value = 0 }; typedef A F; };
template <class A, int M> struct FastSel<AccSel<A, M>> { enum { value = 1 }; typedef AccSelFast<A, M> F; };

// Moments for mean / variance / stddev.  Data are shifted by k (the first
// element of the output's reduction set), then sum(d) and sum(d*d) are
// accumulated — in double-float for float32/bf16 data (TwoSum + exact
// products by fma), in FP64 for float64 data; partial states from different
// blocks combine in FP64.  MODE 0 = mean (k = 0, no second moment),
// 1 = variance, 2 = stddev.
template <class C, int MODE> struct AccMom;
template <int MODE> struct AccMom<float, MODE> {
    float k;
    AccSumC s1, s2;
    template <class P> XTG_DI void init(const P& p);
    template <class X> XTG_DI void add(X x, i64) {
        float d = cvt<float>(x) - k;
        s1.addf(d);
        if (MODE != 0) {
            float q = d * d;
            float qe = fmaf(d, d, -q);
            s2.addf(q);
            s2.lo += qe;
        }
    }
    XTG_DI void merge(const AccMom& o) { s1.merge(o.s1); if (MODE != 0) s2.merge(o.s2); }
};
template <int MODE> struct AccMom<double, MODE> {
    double k, s1, s2;
    template <class P> XTG_DI void init(const P& p);
    template <class X> XTG_DI void add(X x, i64) {
        double d = cvt<double>(x) - k;
        s1 += d;
        if (MODE != 0) s2 = fma(d, d, s2);
    }
    XTG_DI void merge(const AccMom& o) { s1 += o.s1; s2 += o.s2; }
};

// Norms (include/xtensor/reducers/xnorm.hpp:397-437): accumulate in the
// big-promoted type.  NK 0 = l0 (count of non-zeros), 1 = l1 (sum |x|),
// 2 = sq (sum x*x), 3 = linf (max |x| from 0, std::max then math::maximum).
template <class A, int NK> struct AccNorm {
    A s;
    template <class P> XTG_DI void init(const P&) { s = A(0); }
    template <class X> XTG_DI void add(X x, i64) {
        if (NK == 0) s = s + (A)(x != X(0) ? 1 : 0);
        else if (NK == 1) s = s + (A)m_abs(x);
        else if (NK == 2) s = s + (A)(x * x);
        else { A a = (A)m_abs(x); s = (s < a) ? a : s; }
    }
    XTG_DI void merge(const AccNorm& o) {
        if (NK == 3) s = (s > o.s) ? s : o.s; else s = s + o.s;
    }
    XTG_DI double dval() const { return (double)s; }
};
// float32 / bf16 squares and absolute values in double-float.
template <int NK> struct AccNormC {
    AccSumC a;
    template <class P> XTG_DI void init(const P&) { a.hi = 0.f; a.lo = 0.f; }
    template <class X> XTG_DI void add(X x, i64) {
        float f = cvt<float>(x);
        if (NK == 1) {
            a.addf(fabsf(f));
        } else {
            float q = f * f;
            float qe = fmaf(f, f, -q);
            a.addf(q);
            a.lo += qe;
        }
    }
    XTG_DI void merge(const AccNormC& o) { a.merge(o.a); }
    XTG_DI double dval() const { return a.dval(); }
};

// Working accumulators of the row pass for the double-float states above:
// two (hi, lo) lanes, even elements of a vector into lane 0 and odd ones into
// lane 1, each lane updated by TwoSum exactly as the scalar state is, with
// packed instructions (half the issue slots: these loops are issue-bound for
// 2-byte inputs and for the two-sum moments).  from() starts lane 0 at the
// stored state and lane 1 at zero; to() merges lane 1 into lane 0 with the
// TwoSum merge when the work item ends, so partial slots and combines keep
// the stored form.  add() (scalar, lane 0) serves odd vector widths.
struct AccSumC2 {
    float2 hi, lo;
    XTG_DI void from(const AccSumC& a) {
        hi = make_float2(a.hi, 0.f);
        lo = make_float2(a.lo, 0.f);
    }
    XTG_DI void to(AccSumC& a) const {
        a.hi = hi.x;
        a.lo = lo.x;
        AccSumC b;
        b.hi = hi.y;
        b.lo = lo.y;
        a.merge(b);
    }
    XTG_DI void addp(float2 v) {
        float2 s, e;
        two_sum2(hi, v, s, e);
        hi = s;
        lo = p_add(lo, e);
    }
    XTG_DI void adds(float v) {
        float s, e;
        two_sum(hi.x, v, s, e);
        hi.x = s;
        lo.x += e;
    }
    template <class X> XTG_DI void add(X x, i64) { adds(cvt<float>(x)); }
    template <class X> XTG_DI void add2(X x0, X x1, i64) { addp(make_float2(cvt<float>(x0), cvt<float>(x1))); }
    // a vector of 2M values (M pairs): their pairwise sum, then one TwoSum
    template <int M> XTG_DI void addblk(const float2 (&f)[M]) {
        const float2 h = Pw2<M>::sum(f);
        adds(h.x + h.y);
    }
};
// Working form of the float32 moments: one packed double-float pair, lane x
// the sum of deviations from the shift k, lane y the sum of their squares,
// so a single packed TwoSum advances both.
template <int MODE> struct AccMom2 {
    float k;
    float2 hi, lo;
    XTG_DI void from(const AccMom<float, MODE>& a) {
        k = a.k;
        hi = make_float2(a.s1.hi, a.s2.hi);
        lo = make_float2(a.s1.lo, a.s2.lo);
    }
    XTG_DI void to(AccMom<float, MODE>& a) const {
        a.k = k;
        a.s1.hi = hi.x;
        a.s1.lo = lo.x;
        a.s2.hi = hi.y;
        a.s2.lo = lo.y;
    }
    XTG_DI void addp2(float2 v) {
        float2 s, e;
        two_sum2(hi, v, s, e);
        hi = s;
        lo = p_add(lo, e);
    }
    template <class X> XTG_DI void add(X x, i64) {
        const float d = cvt<float>(x) - k;
        const float q = d * d;
        addp2(make_float2(d, q));
        lo.y += fmaf(d, d, -q);  // the square's rounding error (exact)
    }
    template <class X> XTG_DI void add2(X x0, X x1, i64 p0) {
        add(x0, p0);
        add(x1, p0 + 1);
    }
    // a vector of 2M values: pairwise sums of the deviations and of their
    // squares (terms >= 0: relative error <= (ceil(log2 2M) + 1) u), one
    // packed TwoSum for both
    template <int M> XTG_DI void addblk(const float2 (&f)[M]) {
        const float2 kk = make_float2(k, k);
        float2 d[M];
#pragma unroll
        for (int i = 0; i < M; ++i) d[i] = p_sub(f[i], kk);
        const float2 hs = Pw2<M>::sum(d);
        const float2 hq = Pw2<M>::sq(d);
        addp2(make_float2(hs.x + hs.y, hq.x + hq.y));
    }
};
template <int NK> struct AccNormC2 {
    AccSumC2 a;
    XTG_DI void from(const AccNormC<NK>& o) { a.from(o.a); }
    XTG_DI void to(AccNormC<NK>& o) const { a.to(o.a); }
    template <class X> XTG_DI void add(X x, i64) {
        const float f = cvt<float>(x);
        if (NK == 1) {
            a.adds(fabsf(f));
        } else {
            const float q = f * f;
            const float qe = fmaf(f, f, -q);
            a.adds(q);
            a.lo.x += qe;
        }
    }
    template <class X> XTG_DI void add2(X x0, X x1, i64) {
        const float2 f = make_float2(cvt<float>(x0), cvt<float>(x1));
        if (NK == 1) {
            a.addp(make_float2(fabsf(f.x), fabsf(f.y)));
        } else {
            const float2 q = p_mul(f, f);
            const float2 nqe = p_fma(p_sub(make_float2(0.f, 0.f), f), f, q);
            a.addp(q);
            a.lo = p_sub(a.lo, nqe);
        }
    }
    template <int M> XTG_DI void addblk(const float2 (&f)[M]) {
        float2 h;
        if (NK == 1) {
            float2 g[M];
#pragma unroll
            for (int j = 0; j < M; ++j) g[j] = make_float2(fabsf(f[j].x), fabsf(f[j].y));
            h = Pw2<M>::sum(g);
        } else {
            h = Pw2<M>::sq(f);
        }
        a.adds(h.x + h.y);
    }
};
// The working form of a stored accumulator in the row pass.
template <class A> struct Work { enum { packed = 0 }; typedef A T; };
template <> struct Work<AccSumC> { enum { packed = 1 }; typedef AccSumC2 T; };
template <int M> struct Work<AccMom<float, M>> { enum { packed = 1 }; typedef AccMom2<M> T; };
template <int NK> struct Work<AccNormC<NK>> { enum { packed = 1 }; typedef AccNormC2<NK> T; };
template <class A> struct HasAdd2 { enum { value = 0 }; };
template <> struct HasAdd2<AccSumC2> { enum { value = 1 }; };
template <int M> struct HasAdd2<AccMom2<M>> { enum { value = 1 }; };
template <int NK> struct HasAdd2<AccNormC2<NK>> { enum { value = 1 }; };
// One pass for sum, mean, variance and norm_l2 (xtg_reduce_moments): the
// four reducers' accumulators side by side (sum and mean share one), each
// fed exactly what its own reduction feeds it, so each result equals that
// reduction's bit for bit.
struct AccStats {
    AccSumC s;
    AccMom<float, 1> m;
    AccNormC<2> q;
    template <class P> XTG_DI void init(const P& p);
    XTG_DI void merge(const AccStats& o) {
        s.merge(o.s);
        m.merge(o.m);
        q.merge(o.q);
    }
};
struct AccStats2 {
    AccSumC2 s;
    AccMom2<1> m;
    AccNormC2<2> q;
    XTG_DI void from(const AccStats& a) {
        s.from(a.s);
        m.from(a.m);
        q.from(a.q);
    }
    XTG_DI void to(AccStats& a) const {
        s.to(a.s);
        m.to(a.m);
        q.to(a.q);
    }
};
template <> struct Work<AccStats> { enum { packed = 1 }; typedef AccStats2 T; };
template <> struct HasAdd2<AccStats2> { enum { value = 1 }; };

// Vector-blocked working forms: a vector's values are summed pairwise in
// float32 and the block enters the double-float state by one TwoSum (for the
// moments about 21 FP32 instructions per 8 values, packed, instead of 76; for
// sums of 2-byte values about 11 instead of 28: at HBM speed those loops are
// bound by instruction issue and the FP32 pipe).
// Used where the blocks' rounding stays small against the result: the
// moments of variance / stddev and the norms (squares and absolute values:
// every term >= 0, so a block's error is relative to the block's own sum),
// and sums and means of 2-byte inputs (bfloat16: 8 significant bits, so a
// vector's pairwise sum is mostly exact); float32 sums and means keep a
// TwoSum per element (their terms cancel).
template <class W, class X> struct BlockAdd { enum { value = 0 }; };
template <class X> struct BlockAdd<AccSumC2, X> { enum { value = sizeof(X) == 2 }; };
template <int NK, class X> struct BlockAdd<AccNormC2<NK>, X> { enum { value = 1 }; };
template <int M, class X> struct BlockAdd<AccMom2<M>, X> { enum { value = M != 0 || sizeof(X) == 2 }; };

template <class A> struct IsStats2 { enum { value = 0 }; };
template <> struct IsStats2<AccStats2> { enum { value = 1 }; };

// One vector of tree values into an accumulator: in pairs where it takes
// them, else element by element; p0 = the first element's position.
template <bool PAIRS> struct AddVec {
    template <int VEC, class Tree, class A, class RG, class C>
    static XTG_DI void run(A& a, const RG& rg, i64 p0, const C& c) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) a.add(Tree::ev(rg, j, c), p0 + j);
    }
};
template <> struct AddVec<true> {
    template <int VEC, class Tree, class A, class RG, class C>
    static XTG_DI void run(A& a, const RG& rg, i64 p0, const C& c) {
        typedef decltype(Tree::ev(rg, 0, c)) X;
        if constexpr (IsStats2<A>::value) {
            run<VEC, Tree>(a.s, rg, p0, c);
            run<VEC, Tree>(a.m, rg, p0, c);
            run<VEC, Tree>(a.q, rg, p0, c);
        } else if constexpr (BlockAdd<A, X>::value != 0 && VEC > 1) {
            float2 f[VEC / 2];
#pragma unroll
            for (int j = 0; j < VEC / 2; ++j)
                f[j] = make_float2(cvt<float>(Tree::ev(rg, 2 * j, c)), cvt<float>(Tree::ev(rg, 2 * j + 1, c)));
            a.template addblk<VEC / 2>(f);
        } else if (VEC % 2 == 0) {
#pragma unroll
            for (int j = 0; j < VEC; j += 2) a.add2(Tree::ev(rg, j, c), Tree::ev(rg, j + 1, c), p0 + j);
        } else {
#pragma unroll
            for (int j = 0; j < VEC; ++j) a.add(Tree::ev(rg, j, c), p0 + j);
        }
    }
};

// Arg-reductions (include/xtensor/misc/xsort.hpp:1158-1296): strict compare,
// first index wins; NaN never wins unless it is the very first element (the
// reference then returns 0 because nothing compares greater than NaN).
template <class A, int MAXOP> struct AccArg {
    A v;
    i64 idx;  // -1: empty
    template <class P> XTG_DI void init(const P&) { idx = -1; v = A(0); }
    template <class X> XTG_DI void add(X x, i64 ps) {
        A a = cvt<A>(x);
        if (idx < 0) {
            if (a == a || ps == 0) { v = a; idx = ps; }
        } else if (MAXOP ? Cmp<A>::gt(a, v) : Cmp<A>::lt(a, v)) {
            v = a;
            idx = ps;
        }
    }
    // add() once a value is held (idx >= 0): the compare and the selects only
    template <class X> XTG_DI void add_held(X x, i64 ps) {
        A a = cvt<A>(x);
        if (MAXOP ? Cmp<A>::gt(a, v) : Cmp<A>::lt(a, v)) {
            v = a;
            idx = ps;
        }
    }
    // add_held() with the candidate's position kept as a 32-bit offset `ro`
    // from the work item's start, in `bo` (the caller adds the start back)
    template <class X> XTG_DI void add_held_off(X x, u32 ro, u32& bo) {
        A a = cvt<A>(x);
        if (MAXOP ? Cmp<A>::gt(a, v) : Cmp<A>::lt(a, v)) {
            v = a;
            bo = ro;
        }
    }
    XTG_DI bool held() const { return idx >= 0; }
    XTG_DI void merge(const AccArg& o) {
        if (o.idx < 0) return;
        if (idx < 0) { v = o.v; idx = o.idx; return; }
        bool nan_me = !(v == v), nan_o = !(o.v == o.v);
        if (nan_me) return;
        if (nan_o) { v = o.v; idx = o.idx; return; }
        bool take = MAXOP ? Cmp<A>::gt(o.v, v) : Cmp<A>::lt(o.v, v);
        if (!take && !(MAXOP ? Cmp<A>::gt(v, o.v) : Cmp<A>::lt(v, o.v)) && o.idx < idx) take = true;
        if (take) { v = o.v; idx = o.idx; }
    }
};
// float64 arg-reductions on key64.  The empty state holds the end key that
// every non-NaN value beats; a NaN taken as the very first element is held as
// the other end key, which nothing beats.
template <int MAXOP> __device__ __noinline__ KeyPos arg_special(i64 kv, i64 idx, double a, i64 ps) {
    KeyPos r;
    r.k = kv;
    r.p = idx;
    const i64 b = __double_as_longlong(a);
    const bool nan = f64_isnan_bits(b);
    bool take;
    if (idx < 0) take = !nan || ps == 0;
    else take = MAXOP ? (a > unkey64(kv)) : (a < unkey64(kv));
    if (take) {
        r.k = nan ? (MAXOP ? XTG_KEY_MAX : XTG_KEY_MIN) : key64(b);
        r.p = ps;
    }
    return r;
}
template <int MAXOP> struct AccArg<double, MAXOP> {
    i64 kv;
    i64 idx;  // -1: empty
    template <class P> XTG_DI void init(const P&) {
        idx = -1;
        kv = MAXOP ? XTG_KEY_MIN : XTG_KEY_MAX;
    }
    XTG_DI double value() const { return unkey64(kv); }
    // The key compare comes first, non-strict: wherever key order and IEEE
    // order differ for an incoming value a (a = +0 after -0 for argmax, -0
    // after +0 for argmin, a NaN whose key sits at the far end or equals the
    // empty state's end key), a is a candidate by key and special, so the
    // exact path decides.  A NaN whose key sits below the held key is never
    // taken, as the fold never takes a NaN after the first element.  Equal
    // keys of ordinary values keep the first (strict order).
    template <class X> XTG_DI void add(X x, i64 ps) {
        const i64 b = __double_as_longlong(cvt<double>(x));
        const i64 ka = key64(b);
        if (MAXOP ? (ka >= kv) : (ka <= kv)) {
            if (f64_special(b)) {
                const KeyPos r = arg_special<MAXOP>(kv, idx, __longlong_as_double(b), ps);
                kv = r.k;
                idx = r.p;
                return;
            }
            if (ka != kv) {
                kv = ka;
                idx = ps;
            }
        }
    }
    XTG_DI void merge(const AccArg& o) {
        if (o.idx < 0) return;
        if (idx < 0) {
            kv = o.kv;
            idx = o.idx;
            return;
        }
        const double v = value(), ov = o.value();
        const bool nan_me = !(v == v), nan_o = !(ov == ov);
        if (nan_me) return;
        if (nan_o) {
            kv = o.kv;
            idx = o.idx;
            return;
        }
        bool take = MAXOP ? (ov > v) : (ov < v);
        if (!take && !(MAXOP ? (v > ov) : (v < ov)) && o.idx < idx) take = true;
        if (take) {
            kv = o.kv;
            idx = o.idx;
        }
    }
};

// ---------------------------------------------------------------------------
// Reduction parameters.  Output space = kept dims (rank RO), reduced space =
// reduced dims (rank RR).  For the ROW strategy the innermost reduced dim is
// vectorised (rshape[RR-1] counted in vectors); for COL the innermost kept
// dim is (oshape[RO-1] counted in vectors).
template <class A, int OP> template <class P> XTG_DI void AccPlain<A, OP>::init(const P& p) {
    s = IsFloat<A>::value ? (A)p.init_f : (A)p.init_i;
}
template <class P> XTG_DI void AccSumC::init(const P& p) { hi = (float)p.init_f; lo = 0.f; }
template <class A, int MAXOP> template <class P> XTG_DI void AccSel<A, MAXOP>::init(const P& p) {
    v = IsFloat<A>::value ? (A)p.init_f : (A)p.init_i;
    pos = -1;
}
template <int MODE> template <class P> XTG_DI void AccMom<float, MODE>::init(const P&) {
    k = 0.f;
    s1.hi = s1.lo = s2.hi = s2.lo = 0.f;
}
template <int MODE> template <class P> XTG_DI void AccMom<double, MODE>::init(const P&) { k = 0.0; s1 = s2 = 0.0; }
template <class P> XTG_DI void AccStats::init(const P& p) {
    s.init(p);
    m.init(p);
    q.init(p);
}

// Shift for the moment accumulators (the output's first element).
template <class A> struct Shift {
    template <class X> static XTG_DI void set(A&, X) {}
};
template <int MODE> struct Shift<AccMom<float, MODE>> {
    template <class X> static XTG_DI void set(AccMom<float, MODE>& a, X x) { a.k = MODE == 0 ? 0.f : cvt<float>(x); }
};
template <int MODE> struct Shift<AccMom<double, MODE>> {
    template <class X> static XTG_DI void set(AccMom<double, MODE>& a, X x) { a.k = MODE == 0 ? 0.0 : cvt<double>(x); }
};
template <> struct Shift<AccStats> {
    template <class X> static XTG_DI void set(AccStats& a, X x) { Shift<AccMom<float, 1>>::set(a.m, x); }
};
template <class A> struct NeedsShift { enum { value = 0 }; };
template <> struct NeedsShift<AccStats> { enum { value = 1 }; };
template <int MODE> struct NeedsShift<AccMom<float, MODE>> { enum { value = MODE != 0 }; };
template <int MODE> struct NeedsShift<AccMom<double, MODE>> { enum { value = MODE != 0 }; };
// arg-reductions whose update has a cheaper form once a value is held
// (float64 keeps its key path)
template <class A> struct HeldFast { enum { value = 0 }; };
template <class A, int M> struct HeldFast<AccArg<A, M>> { enum { value = 1 }; };
template <int M> struct HeldFast<AccArg<double, M>> { enum { value = 0 }; };
// one step of a column walk: VEC accumulators take row r of their columns.
// Until every one of them holds a value the full update runs; after that
// (held == true) the compare-and-select form.
template <class Tree, class Acc, int VEC> struct ColStep {
    template <class RG, class C>
    static XTG_DI void run(Acc (&acc)[VEC], const RG& rg, i64 r, const C& c, bool& held) {
        if constexpr (HeldFast<Acc>::value) {
            if (held) {
#pragma unroll
                for (int j = 0; j < VEC; ++j) acc[j].add_held(Tree::ev(rg, j, c), r);
                return;
            }
            bool h = true;
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                acc[j].add(Tree::ev(rg, j, c), r);
                h = h && acc[j].held();
            }
            held = h;
        } else {
#pragma unroll
            for (int j = 0; j < VEC; ++j) acc[j].add(Tree::ev(rg, j, c), r);
        }
    }
};

// Finalisation: accumulator state -> output element (merging xt::initial
// last, as xreducer_stepper::aggregate does, xreducer.hpp:1778-1799).
template <class Out, class A> struct Fin;
template <class Out, class A, int OP> struct Fin<Out, AccPlain<A, OP>> {
    template <class P> static XTG_DI Out go(const AccPlain<A, OP>& a, const P& p) {
        A r = a.s;
        if (p.has_initial) {
            A iv = IsFloat<A>::value ? (A)p.initial_f : (A)p.initial_i;
            r = OP == 0 ? (A)(iv + r) : (A)(iv * r);
        }
        return cvt<Out>(r);
    }
};
template <class Out> struct Fin<Out, AccSumC> {
    template <class P> static XTG_DI Out go(const AccSumC& a, const P& p) {
        double r = a.dval();
        if (p.has_initial) r = p.initial_f + r;
        return cvt<Out>(r);
    }
};
template <class Out, class A, int MAXOP> struct Fin<Out, AccSel<A, MAXOP>> {
    template <class P> static XTG_DI Out go(const AccSel<A, MAXOP>& a, const P& p) {
        A r = a.value();
        if (p.has_initial) {
            A iv = IsFloat<A>::value ? (A)p.initial_f : (A)p.initial_i;
            r = MAXOP ? (iv > r ? iv : r) : (iv < r ? iv : r);
        }
        return cvt<Out>(r);
    }
};
// mean: sum / divisor in double (mean_division, xmath.hpp:1828-1835);
// variance: (sum d^2 - (sum d)^2 / n) / divisor; stddev: sqrt of that.
template <int MODE> XTG_DI void mom_sums(const AccMom<float, MODE>& a, double& s1, double& s2) {
    s1 = a.s1.dval();
    s2 = a.s2.dval();
}
template <int MODE> XTG_DI void mom_sums(const AccMom<double, MODE>& a, double& s1, double& s2) {
    s1 = a.s1;
    s2 = a.s2;
}
template <class Out, class C, int MODE> struct Fin<Out, AccMom<C, MODE>> {
    template <class P> static XTG_DI Out go(const AccMom<C, MODE>& a, const P& p) {
        double s1, s2;
        mom_sums(a, s1, s2);
        if (MODE == 0) return cvt<Out>(s1 / p.divisor);
        double n = (double)p.n_red;
        double m2 = s2 - s1 * (s1 / n);
        if (m2 < 0.0) m2 = 0.0;
        double var = m2 / p.divisor;
        return cvt<Out>(MODE == 2 ? sqrt(var) : var);
    }
};
template <class Out, class A, int NK> struct Fin<Out, AccNorm<A, NK>> {
    template <class P> static XTG_DI Out go(const AccNorm<A, NK>& a, const P&) { return cvt<Out>(a.s); }
};
template <class Out, int NK> struct Fin<Out, AccNormC<NK>> {
    template <class P> static XTG_DI Out go(const AccNormC<NK>& a, const P&) { return cvt<Out>(a.dval()); }
};
template <class Out, class A, int MAXOP> struct Fin<Out, AccArg<A, MAXOP>> {
    template <class P> static XTG_DI Out go(const AccArg<A, MAXOP>& a, const P&) { return cvt<Out>(a.idx < 0 ? 0 : a.idx); }
};
// Post-processing applied after Fin: POST 1 = sqrt (norm_l2 = sqrt(norm_sq),
// include/xtensor/reducers/xnorm.hpp:494-526); POST 2 = division by the
// mean divisor in double (mean_division, include/xtensor/core/xmath.hpp:1828-1835).
template <int POST, class Out, class V, class P> XTG_DI Out post(V v, const P& p) {
    if (POST == 1) return cvt<Out>(m_sqrt(cvt<double>(v)));
    if (POST == 2) return cvt<Out>(cvt<double>(v) / p.divisor);
    return cvt<Out>(v);
}
// Value type handed from Fin to post: POST 2 keeps the sum in double.
template <int POST, class Out> struct FinT { typedef Out type; };
template <class Out> struct FinT<2, Out> { typedef double type; };
template <class Out, class Acc, int POST, class P> XTG_DI Out finish(const Acc& a, const P& p) {
    typedef typename FinT<POST, Out>::type M;
    return post<POST, Out>(Fin<M, Acc>::go(a, p), p);
}
// A reduction's result(s) at output offset oo.
template <class TS, class TM, class TV, class TN> struct StatsOut {};
template <class Out, class Acc, int POST> struct Store {
    static XTG_DI void put(const Acc& a, const RedParams& p, i64 oo) {
        reinterpret_cast<Out*>(p.out)[oo] = finish<Out, Acc, POST>(a, p);
    }
};
template <class TS, class TM, class TV, class TN, int POST> struct Store<StatsOut<TS, TM, TV, TN>, AccStats, POST> {
    static XTG_DI void put(const AccStats& a, const RedParams& p, i64 oo) {
        FinP pm;  // what the finishers read: no initial value, the mean's divisor
        pm.init_f = 0.0;
        pm.init_i = 0;
        pm.has_initial = 0;
        pm.initial_f = 0.0;
        pm.initial_i = 0;
        pm.divisor = p.divisor;
        pm.n_red = p.n_red;
        FinP pv = pm;  // the variance's divisor
        pv.divisor = p.divisor2;
        if (p.out) reinterpret_cast<TS*>(p.out)[oo] = finish<TS, AccSumC, 0>(a.s, pm);
        if (p.out_more[0]) reinterpret_cast<TM*>(p.out_more[0])[oo] = finish<TM, AccSumC, 2>(a.s, pm);
        if (p.out_more[1]) reinterpret_cast<TV*>(p.out_more[1])[oo] = finish<TV, AccMom<float, 1>, 0>(a.m, pv);
        if (p.out_more[2]) reinterpret_cast<TN*>(p.out_more[2])[oo] = finish<TN, AccNormC<2>, 1>(a.q, pm);
    }
};

// Offsets of every leaf at a (kept, reduced) multi-index pair.
template <int NL, int RO, int RR>
XTG_DI void red_offsets(const RedParams& p, const i64 (&ko)[RO], const i64 (&ro)[RR], i64 (&off)[XTG_KMAX_LEAVES]) {
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        i64 o = 0;
#pragma unroll
        for (int d = 0; d < RO; ++d) o += ko[d] * p.lks[l][d];
#pragma unroll
        for (int d = 0; d < RR; ++d) o += ro[d] * p.lrs[l][d];
        off[l] = o;
    }
}

template <int R, bool BIG>
XTG_DI void decode_dims(const i64* shape, const FastDiv* fd, i64 q, i64 (&idx)[R]) {
    if (BIG || R == 1) {
#pragma unroll
        for (int d = R - 1; d >= 1; --d) {
            i64 n = shape[d];
            i64 qq = q / n;
            idx[d] = q - qq * n;
            q = qq;
        }
        idx[0] = q;
    } else {
        u32 qu = (u32)q;
#pragma unroll
        for (int d = R - 1; d >= 1; --d) {
            u32 qq = fdiv(qu, fd[d]);
            idx[d] = qu - qq * fd[d].d;
            qu = qq;
        }
        idx[0] = qu;
    }
}

// Loads of all leaves at explicit offsets (vector along a given inner stride).
template <int I, int VEC, class... S> struct LoadAt;
template <int I, int VEC> struct LoadAt<I, VEC> {
    template <class RG> static XTG_DI void run(RG&, const void* const*, const i64*, const i64*) {}
};
template <int I, int VEC, class S0, class... S> struct LoadAt<I, VEC, S0, S...> {
    template <class RG> static XTG_DI void run(RG& rg, const void* const* ptr, const i64* off, const i64* inner) {
        typedef typename S0::type T;
        ld_leaf<T, S0::kind, VEC>(rg.v, reinterpret_cast<const T*>(ptr[I]), off[I], inner[I]);
        LoadAt<I + 1, VEC, S...>::run(rg.rest, ptr, off, inner);
    }
};
template <class LS> struct LoadLeavesAt;
template <class... S> struct LoadLeavesAt<LeafSet<S...>> {
    template <int VEC, class RG> static XTG_DI void run(RG& rg, const void* const* ptr, const i64* off, const i64* inner) {
        LoadAt<0, VEC, S...>::run(rg, ptr, off, inner);
    }
};
// All leaves but leaf 0 (the transposing kernel fills leaf 0 from shared memory).
template <class LS> struct LoadRest;
template <class S0, class... S> struct LoadRest<LeafSet<S0, S...>> {
    template <class RG> static XTG_DI void run(RG& rg, const void* const* ptr, const i64* off, const i64* inner) {
        LoadAt<1, 1, S...>::run(rg.rest, ptr, off, inner);
    }
};

// Asynchronous global -> shared copies of 4, 8 or 16 bytes (cp.async): the
// copies are in flight without holding registers; a thread's own copies are
// visible to it after cp.async.wait_group.
XTG_DI unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
template <int B> XTG_DI void cp_async(void* dst, const void* src) {
    if (B == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
    else if (B == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
XTG_DI void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> XTG_DI void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Per-leaf ring slots of the COL kernel: slot (stage, leaf, thread) is 16
// bytes at ((stage * NL + leaf) * blockDim + thread) * 16.
template <int I, int VEC, class... S> struct RingAt;
template <int I, int VEC> struct RingAt<I, VEC> {
    static XTG_DI void issue(unsigned char*, int, const void* const*, const i64*) {}
    template <class RG> static XTG_DI void read(RG&, const unsigned char*, int) {}
};
template <int I, int VEC, class S0, class... S> struct RingAt<I, VEC, S0, S...> {
    typedef typename S0::type T;
    static XTG_DI void issue(unsigned char* slot0, int lstride, const void* const* ptr, const i64* off) {
        cp_async<(int)sizeof(T) * VEC>(slot0 + (size_t)I * lstride, reinterpret_cast<const T*>(ptr[I]) + off[I]);
        RingAt<I + 1, VEC, S...>::issue(slot0, lstride, ptr, off);
    }
    template <class RG> static XTG_DI void read(RG& rg, const unsigned char* slot0, int lstride) {
        constexpr int B = (int)sizeof(T) * VEC;
        typedef typename VecT<B>::t V;
        union { V v; T e[VEC]; } u;
        u.v = *reinterpret_cast<const V*>(slot0 + (size_t)I * lstride);
#pragma unroll
        for (int j = 0; j < VEC; ++j) rg.v[j] = u.e[j];
        RingAt<I + 1, VEC, S...>::read(rg.rest, slot0, lstride);
    }
};
template <class LS, int VEC> struct Ring;
template <class... S, int VEC> struct Ring<LeafSet<S...>, VEC> {
    static XTG_DI void issue(unsigned char* slot0, int lstride, const void* const* ptr, const i64* off) {
        RingAt<0, VEC, S...>::issue(slot0, lstride, ptr, off);
    }
    template <class RG> static XTG_DI void read(RG& rg, const unsigned char* slot0, int lstride) {
        RingAt<0, VEC, S...>::read(rg, slot0, lstride);
    }
};

// K3/K5: ROW strategy — the reduced run is contiguous (or broadcast) for the
// leaves; a group (warp or CTA) owns one (output, split) work item and strides
// over its vectors.  Work items: w = o * nsplit + s.
// The values of an evaluated vector as a tree (fused assign + reduce: the
// accumulator takes the values exactly as they were stored).
struct ArrVal {
    template <class RG, class C> static XTG_DI auto ev(const RG& r, int j, const C&) { return r[j]; }
};
// ES: 0 reduce only; 1 also store each evaluated vector, contiguous and
// aligned, into p.eout (type ET); 2 the same with element-wise strided stores.
// PK: 1 = the packed working accumulator (Work<Acc>) for double-float
// states, 0 = the stored state's own add.
template <class Tree, class LS, class Acc, class Out, int POST, int VEC, int RO, int RR, int GROUP, bool BIG, int UR = 4,
          int ES = 0, class ET = float, int PK = 1>
__global__ void __launch_bounds__(256) k_reduce_row(const RedParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    __shared__ Acc smem[32];
    Ctx<0> c;
    c.scal = p.scal;
    const int gsz = GROUP <= 32 ? 32 : (int)blockDim.x;
    const int groups_per_block = (int)blockDim.x / gsz;
    const int gtid = (int)threadIdx.x % gsz;
    const i64 gid = (i64)blockIdx.x * groups_per_block + (int)threadIdx.x / gsz;
    const i64 ngroups = (i64)gridDim.x * groups_per_block;
    const i64 nwork = p.n_out * p.nsplit;
    i64 inner[XTG_KMAX_LEAVES];
#pragma unroll
    for (int l = 0; l < LS::N; ++l) inner[l] = p.lrs[l][RR - 1];
    for (i64 w = gid; w < nwork; w += ngroups) {
        const i64 o = p.nsplit == 1 ? w : w / p.nsplit;
        const i64 s = w - o * p.nsplit;
        i64 ko[RO];
        // 32-bit multiply-shift division when the outputs fit (the host sets
        // every ofd), 64-bit division otherwise
        if (p.n_out <= 0xFFFFFFF0ll) decode_dims<RO, false>(p.oshape, p.ofd, o, ko);
        else decode_dims<RO, true>(p.oshape, p.ofd, o, ko);
        Acc acc;
        acc.init(p);
        if (NeedsShift<Acc>::value && p.n_red > 0) {
            i64 r0[RR];
#pragma unroll
            for (int d = 0; d < RR; ++d) r0[d] = 0;
            i64 off[XTG_KMAX_LEAVES];
            red_offsets<LS::N, RO, RR>(p, ko, r0, off);
            typename LS::template R<1>::type rg1;
            LoadLeavesAt<LS>::template run<1>(rg1, p.leaf, off, inner);
            Shift<Acc>::set(acc, Tree::ev(rg1, 0, c));
        }
        const i64 rb = s * p.chunk;
        i64 re = rb + p.chunk;
        if (re > p.n_redv) re = p.n_redv;
        // each leaf's (and the fused destination's) offset of the output
        // position, once per work item: the vectors add the reduced part only
        i64 kbase[XTG_KMAX_LEAVES];
#pragma unroll
        for (int l = 0; l < LS::N; ++l) {
            i64 o = 0;
#pragma unroll
            for (int d = 0; d < RO; ++d) o += ko[d] * p.lks[l][d];
            kbase[l] = o;
        }
        i64 ebase = 0;
        if constexpr (ES != 0) {
#pragma unroll
            for (int d = 0; d < RO; ++d) ebase += ko[d] * p.eks[d];
        }
        // two register batches of U vectors: the next batch's loads are in
        // flight while the current one is reduced; each thread still visits
        // its positions in increasing order
        constexpr int U = UR;
        const i64 step = (i64)gsz * U;
        RG rga[U], rgb[U];
        auto load = [&](RG(&rg)[U], i64 r0) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const i64 r = r0 + (i64)u * gsz;
                if (r < re) {
                    i64 ri[RR];
                    decode_dims<RR, BIG>(p.rshape, p.rfd, r, ri);
                    ri[RR - 1] *= VEC;
                    i64 off[XTG_KMAX_LEAVES];
#pragma unroll
                    for (int l = 0; l < LS::N; ++l) {
                        i64 o = kbase[l];
#pragma unroll
                        for (int d = 0; d < RR; ++d) o += ri[d] * p.lrs[l][d];
                        off[l] = o;
                    }
                    LoadLeavesAt<LS>::template run<VEC>(rg[u], p.leaf, off, inner);
                }
            }
        };
// the reduction pass over the work item, folding into accumulator A
#define XTG_ROW_PASS(A)                                                                \
    {                                                                                  \
        auto consume = [&](const RG(&rg)[U], i64 r0) {                                 \
            _Pragma("unroll") for (int u = 0; u < U; ++u) {                            \
                const i64 r = r0 + (i64)u * gsz;                                       \
                if (r < re) {                                                          \
                    if constexpr (ES != 0) {                                           \
                        ET ev[VEC];                                                    \
                        _Pragma("unroll") for (int j = 0; j < VEC; ++j)                \
                            ev[j] = cvt<ET>(Tree::ev(rg[u], j, c));                    \
                        i64 ri[RR];                                                    \
                        decode_dims<RR, BIG>(p.rshape, p.rfd, r, ri);                  \
                        ri[RR - 1] *= VEC;                                             \
                        i64 eo = ebase;                                                \
                        _Pragma("unroll") for (int d = 0; d < RR; ++d) eo += ri[d] * p.ers[d]; \
                        st_out<ET, ES == 1 ? K_CONTIG : 2, VEC>(reinterpret_cast<ET*>(p.eout), eo, \
                                                                 p.ers[RR - 1], ev);   \
                        AddVec<HasAdd2<decltype(A)>::value != 0>::template run<VEC, ArrVal>( \
                            A, ev, r * VEC, c);                                        \
                    } else {                                                           \
                        AddVec<HasAdd2<decltype(A)>::value != 0>::template run<VEC, Tree>( \
                            A, rg[u], r * VEC, c);                                     \
                    }                                                                  \
                }                                                                      \
            }                                                                          \
        };                                                                             \
        i64 r0 = rb + gtid;                                                            \
        if (r0 < re) load(rga, r0);                                                    \
        for (; r0 < re; r0 += 2 * step) {                                              \
            if (r0 + step < re) load(rgb, r0 + step);                                  \
            consume(rga, r0);                                                          \
            if (r0 + step >= re) break;                                                \
            if (r0 + 2 * step < re) load(rga, r0 + 2 * step);                          \
            consume(rgb, r0 + step);                                                   \
        }                                                                              \
    }
        if constexpr (FastSel<Acc>::value && ES == 0) {
            // amax / amin: a position-free pass; the exact pass with
            // positions only when some thread of the group met a NaN, a zero
            // or (float64) another special value
            typename FastSel<Acc>::F fa;
            fa.init(p);
            XTG_ROW_PASS(fa)
            bool ex = fa.exact();
            if (GROUP <= 32) ex = __any_sync(0xffffffffu, ex);
            else ex = __syncthreads_or(ex) != 0;
            if (ex) XTG_ROW_PASS(acc)
            else fa.to(acc);
        } else if constexpr (Work<Acc>::packed != 0 && PK != 0) {
            // double-float states: two lanes advanced by packed instructions
            typename Work<Acc>::T wa;
            wa.from(acc);
            XTG_ROW_PASS(wa)
            wa.to(acc);
        } else {
            XTG_ROW_PASS(acc)
        }
#undef XTG_ROW_PASS
        acc = group_reduce<GROUP>(acc, smem);
        if (gtid == 0) {
            if (p.nsplit > 1) {
                static_assert(sizeof(Acc) <= 32, "split partial slots are 32 bytes");
                reinterpret_cast<Acc*>(p.partial)[w] = acc;
            } else {
                i64 oo = 0;
#pragma unroll
                for (int d = 0; d < RO; ++d) oo += ko[d] * p.ostr[d];
                reinterpret_cast<Out*>(p.out)[oo] = finish<Out, Acc, POST>(acc, p);
            }
        }
        if (GROUP > 32) __syncthreads();
    }
}

// K4: COL strategy — the innermost kept dim is contiguous; each thread owns
// VEC consecutive outputs and walks the reduced space (U loads in flight).
// With RS > 0 (every leaf contiguous along the outputs, VEC * size of 4, 8
// or 16 bytes) the loads are asynchronous copies into a per-thread ring of
// RS stages in shared memory: RS - 1 rows in flight without registers.
// Work items: w = s * n_outv + ov (consecutive threads -> consecutive outputs).
template <class Tree, class LS, class Acc, class Out, int POST, int VEC, int RO, int RR, int U, bool BIG, int RS = 0>
__global__ void __launch_bounds__(256) k_reduce_col(const RedParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    extern __shared__ __align__(16) unsigned char col_ring[];
    Ctx<0> c;
    c.scal = p.scal;
    const i64 nwork = p.n_outv * p.nsplit;
    i64 inner[XTG_KMAX_LEAVES];
#pragma unroll
    for (int l = 0; l < LS::N; ++l) inner[l] = p.lks[l][RO - 1];
    for (i64 w = (i64)blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += (i64)gridDim.x * blockDim.x) {
        const i64 s = w / p.n_outv;
        const i64 ov = w - s * p.n_outv;
        i64 ko[RO];
        decode_dims<RO, BIG>(p.oshape, p.ofd, ov, ko);
        ko[RO - 1] *= VEC;
        Acc acc[VEC];
#pragma unroll
        for (int j = 0; j < VEC; ++j) acc[j].init(p);
        if (NeedsShift<Acc>::value && p.n_red > 0) {
            i64 r0[RR];
#pragma unroll
            for (int d = 0; d < RR; ++d) r0[d] = 0;
            i64 off[XTG_KMAX_LEAVES];
            red_offsets<LS::N, RO, RR>(p, ko, r0, off);
            RG rg;
            LoadLeavesAt<LS>::template run<VEC>(rg, p.leaf, off, inner);
#pragma unroll
            for (int j = 0; j < VEC; ++j) Shift<Acc>::set(acc[j], Tree::ev(rg, j, c));
        }
        const i64 rb = s * p.chunk;
        i64 re = rb + p.chunk;
        if (re > p.n_redv) re = p.n_redv;
        bool held = false;
        // each leaf's offset of the output position, once per work item
        i64 kbase[XTG_KMAX_LEAVES];
#pragma unroll
        for (int l = 0; l < LS::N; ++l) {
            i64 o = 0;
#pragma unroll
            for (int d = 0; d < RO; ++d) o += ko[d] * p.lks[l][d];
            kbase[l] = o;
        }
        auto offsets = [&](i64 r, i64(&off)[XTG_KMAX_LEAVES]) {
            i64 ri[RR];
            decode_dims<RR, BIG>(p.rshape, p.rfd, r, ri);
#pragma unroll
            for (int l = 0; l < LS::N; ++l) {
                i64 o = kbase[l];
#pragma unroll
                for (int d = 0; d < RR; ++d) o += ri[d] * p.lrs[l][d];
                off[l] = o;
            }
        };

        if constexpr (RS > 0) {
            const int lstride = (int)blockDim.x * 16;
            const int sstride = LS::N * lstride;
            unsigned char* mine = col_ring + (size_t)threadIdx.x * 16;
            auto issue = [&](i64 r, int st) {
                i64 off[XTG_KMAX_LEAVES];
                offsets(r, off);
                Ring<LS, VEC>::issue(mine + (size_t)st * sstride, lstride, p.leaf, off);
            };
#pragma unroll
            for (int k = 0; k < RS - 1; ++k) {
                if (rb + k < re) issue(rb + k, k);
                cp_async_commit();
            }
            int st = 0;
            // held arg-updates keep the best position as a 32-bit offset from
            // rb (one select instead of two per element) when the item allows
            u32 bo[VEC];
            bool h32 = false;
            const bool can32 = re - rb <= (i64)0xFFFFFFFF;
            for (i64 r = rb; r < re; ++r) {
                cp_async_wait<RS - 2>();  // row r's copies have landed
                RG rg;
                Ring<LS, VEC>::read(rg, mine + (size_t)st * sstride, lstride);
                // refill the slot row r - 1 used (read in the previous step)
                const int sf = st == 0 ? RS - 1 : st - 1;
                if (r + RS - 1 < re) issue(r + RS - 1, sf);
                cp_async_commit();
                if constexpr (HeldFast<Acc>::value) {
                    if (h32) {
                        const u32 ro = (u32)(r - rb);
#pragma unroll
                        for (int j = 0; j < VEC; ++j) acc[j].add_held_off(Tree::ev(rg, j, c), ro, bo[j]);
                    } else {
                        ColStep<Tree, Acc, VEC>::run(acc, rg, r, c, held);
                        if (held && can32) {
                            h32 = true;
#pragma unroll
                            for (int j = 0; j < VEC; ++j) bo[j] = (u32)(acc[j].idx - rb);
                        }
                    }
                } else {
                    ColStep<Tree, Acc, VEC>::run(acc, rg, r, c, held);
                }
                st = st == RS - 1 ? 0 : st + 1;
            }
            if constexpr (HeldFast<Acc>::value) {
                if (h32) {
#pragma unroll
                    for (int j = 0; j < VEC; ++j) acc[j].idx = rb + (i64)bo[j];
                }
            }
            cp_async_wait<0>();
        } else {
        for (i64 r = rb; r < re; r += U) {
            RG rg[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (r + u < re) {
                    i64 off[XTG_KMAX_LEAVES];
                    offsets(r + u, off);
                    LoadLeavesAt<LS>::template run<VEC>(rg[u], p.leaf, off, inner);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (r + u < re) ColStep<Tree, Acc, VEC>::run(acc, rg[u], r + u, c, held);
            }
        }
        }
        // flat output index of the first of the VEC outputs
        i64 ofl = 0;
#pragma unroll
        for (int d = 0; d < RO; ++d) ofl = ofl * (d == RO - 1 ? p.oshape[d] * VEC : p.oshape[d]) + ko[d];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            if (p.nsplit > 1) {
                reinterpret_cast<Acc*>(p.partial)[(ofl + j) * p.nsplit + s] = acc[j];
            } else {
                i64 oo = 0;
#pragma unroll
                for (int d = 0; d < RO; ++d) oo += ko[d] * p.ostr[d];
                oo += (i64)j * p.ostr[RO - 1];
                reinterpret_cast<Out*>(p.out)[oo] = finish<Out, Acc, POST>(acc[j], p);
            }
        }
    }
}

// Combine for few splits per output: one thread per output merges its
// partials in split order.
template <class Acc, class Out, int POST, int RO>
__global__ void __launch_bounds__(256) k_reduce_combine_thread(const RedParams p) {
    pdl_wait();
    const Acc* part = reinterpret_cast<const Acc*>(p.partial);
    for (i64 o = (i64)blockIdx.x * blockDim.x + threadIdx.x; o < p.n_out; o += (i64)gridDim.x * blockDim.x) {
        Acc a = part[o * p.nsplit];
        for (i64 s = 1; s < p.nsplit; ++s) a.merge(part[o * p.nsplit + s]);
        i64 ko[RO];
        decode_dims<RO, true>(p.oshape, p.ofd, o, ko);
        i64 oo = 0;
#pragma unroll
        for (int d = 0; d < RO; ++d) oo += ko[d] * p.ostr[d];
        Store<Out, Acc, POST>::put(a, p, oo);
    }
}

// Deterministic combine of split partials: one CTA per output, threads take
// splits t, t+blockDim, … in order, then a fixed block tree.
template <class Acc, class Out, int POST, int RO>
__global__ void __launch_bounds__(256) k_reduce_combine(const RedParams p) {
    pdl_wait();
    __shared__ Acc smem[32];
    const Acc* part = reinterpret_cast<const Acc*>(p.partial);
    for (i64 o = blockIdx.x; o < p.n_out; o += gridDim.x) {
        Acc a;
        a.init(p);
        for (i64 s = threadIdx.x; s < p.nsplit; s += blockDim.x) {
            if (s == (i64)threadIdx.x) a = part[o * p.nsplit + s];
            else a.merge(part[o * p.nsplit + s]);
        }
        a = group_reduce<256>(a, smem);
        if (threadIdx.x == 0) {
            i64 ko[RO];
            decode_dims<RO, true>(p.oshape, p.ofd, o, ko);
            i64 oo = 0;
#pragma unroll
            for (int d = 0; d < RO; ++d) oo += ko[d] * p.ostr[d];
            Store<Out, Acc, POST>::put(a, p, oo);
        }
        __syncthreads();
    }
}


// ---------------------------------------------------------------------------
// K9: accumulators — cumsum / cumprod / nancumsum / nancumprod
// (include/xtensor/reducers/xaccumulator.hpp:202-310,
// include/xtensor/core/xmath.hpp:2248-2301, 2363-2391, 2592-2645).  Elements
// are converted to the accumulation type RT, then folded: OP 0 plus,
// 1 multiplies, 2 / 3 the same skipping NaN operands (the first element goes
// through nan_init: NaN -> 0 / 1).
template <class T> XTG_DI bool is_nan_v(T x) { return IsFloat<T>::value && !(x == x); }
template <class RT, int OP> struct ScanOp {
    static XTG_DI RT init(RT x) {
        if (OP >= 2 && is_nan_v(x)) return RT(OP == 2 ? 0 : 1);
        return x;
    }
    static XTG_DI RT step(RT a, RT x) {
        if (OP >= 2 && is_nan_v(x)) return a;
        return (OP & 1) ? RT(a * x) : RT(a + x);
    }
};

// K9a: along a non-innermost axis.  A thread owns VEC adjacent inner
// positions of one outer index and walks the axis in order (U positions'
// loads in flight), so every output element is folded in the reference's
// sequential order.
template <class Tree, class LS, class RT, int OP, int VEC, int OKIND, int U>
__global__ void __launch_bounds__(256) k_scan_col(const ScanParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    Ctx<0> c;
    c.scal = p.scal;
    const i64 nvi = p.n_inner / VEC;
    const i64 nwork = p.n_outer * nvi;
    for (i64 w = (i64)blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += (i64)gridDim.x * blockDim.x) {
        const i64 o = w / nvi, iv = w - o * nvi;
        i64 off[XTG_KMAX_LEAVES], inner[XTG_KMAX_LEAVES];
#pragma unroll
        for (int l = 0; l < LS::N; ++l) {
            off[l] = o * p.lso[l] + iv * VEC * p.lsi[l];
            inner[l] = p.lsi[l];
        }
        i64 oo = o * p.oso + iv * VEC * p.osi;
        RT acc[VEC];
        for (i64 k0 = 0; k0 < p.len; k0 += U) {
            RG rg[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (k0 + u < p.len) {
                    i64 o2[XTG_KMAX_LEAVES];
#pragma unroll
                    for (int l = 0; l < LS::N; ++l) o2[l] = off[l] + (i64)u * p.lsa[l];
                    LoadLeavesAt<LS>::template run<VEC>(rg[u], p.leaf, o2, inner);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (k0 + u < p.len) {
                    RT v[VEC];
#pragma unroll
                    for (int j = 0; j < VEC; ++j) {
                        const RT x = cvt<RT>(Tree::ev(rg[u], j, c));
                        acc[j] = (k0 + u == 0) ? ScanOp<RT, OP>::init(x) : ScanOp<RT, OP>::step(acc[j], x);
                        v[j] = acc[j];
                    }
                    st_out<RT, OKIND, VEC>(reinterpret_cast<RT*>(p.out), oo + (i64)u * p.osa, p.osi, v);
                }
            }
#pragma unroll
            for (int l = 0; l < LS::N; ++l) off[l] += (i64)U * p.lsa[l];
            oo += (i64)U * p.osa;
        }
    }
}

// K9b: along the innermost axis of many rows.  A warp owns 32 rows and walks
// them in chunks of 32*VEC columns: each lane loads VEC adjacent columns of
// every row (16-byte accesses, coalesced), the chunk is transposed through
// shared memory, lane i folds row i's elements in order, and the chunk goes
// back the same way.  Sequential order per row (bit-identical to the
// reference's fold).  VEC > 1 needs rows whose length and starts are
// multiples of VEC (the host checks).
template <class Tree, class LS, class RT, int OP, int VEC, bool RAW = false>
__global__ void __launch_bounds__(64) k_scan_rows(const ScanParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    constexpr int CW = 32 * VEC;        // columns per chunk
    constexpr int RS = CW + VEC;        // padded row stride (keeps 16-byte rows)
    __shared__ __align__(16) RT tile[2][32 * RS];
    Ctx<0> c;
    c.scal = p.scal;
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    RT* tw = tile[warp];
    const i64 ngroups = (p.n_outer + 31) / 32;
    for (i64 g = (i64)blockIdx.x * 2 + warp; g < ngroups; g += (i64)gridDim.x * 2) {
        const i64 r0 = g * 32;
        RT acc = RT(0);
        for (i64 c0 = 0; c0 < p.len; c0 += CW) {
            const i64 col = c0 + (i64)lane * VEC;
            if constexpr (RAW) {
                // the operand is the accumulation type, contiguous along the
                // rows: copy it into the tile, every row's vector in flight
                const RT* src = reinterpret_cast<const RT*>(p.leaf[0]);
#pragma unroll 8
                for (int i = 0; i < 32; ++i) {
                    const i64 r = r0 + i;
                    if (r < p.n_outer && col < p.len)
                        cp_async<(int)sizeof(RT) * VEC>(tw + (i64)i * RS + lane * VEC, src + r * p.lso[0] + col);
                }
                cp_async_commit();
                cp_async_wait<0>();
            } else {
#pragma unroll 4
            for (int i = 0; i < 32; ++i) {
                const i64 r = r0 + i;
                if (r < p.n_outer && col < p.len) {
                    i64 off[XTG_KMAX_LEAVES];
#pragma unroll
                    for (int l = 0; l < LS::N; ++l) off[l] = r * p.lso[l] + col * p.lsa[l];
                    RG rg;
                    LoadLeavesAt<LS>::template run<VEC>(rg, p.leaf, off, p.lsa);
                    RT v[VEC];
#pragma unroll
                    for (int j = 0; j < VEC; ++j) v[j] = cvt<RT>(Tree::ev(rg, j, c));
                    st_out<RT, K_CONTIG, VEC>(tw, (i64)i * RS + lane * VEC, 1, v);
                }
            }
            }
            __syncwarp();
            const int lim = (p.len - c0) < CW ? (int)(p.len - c0) : CW;
            typedef typename VecT<(int)sizeof(RT) * VEC>::t VV;  // VEC * sizeof(RT) <= 16
            union VU {
                VV vv;
                RT e[VEC];
            };
            if (r0 + lane < p.n_outer) {
                RT* row = tw + lane * RS;
                for (int k = 0; k < lim; k += VEC) {
                    VU u;
                    u.vv = *reinterpret_cast<const VV*>(row + k);
#pragma unroll
                    for (int j = 0; j < VEC; ++j) {
                        acc = (c0 + k + j == 0) ? ScanOp<RT, OP>::init(u.e[j]) : ScanOp<RT, OP>::step(acc, u.e[j]);
                        u.e[j] = acc;
                    }
                    *reinterpret_cast<VV*>(row + k) = u.vv;
                }
            }
            __syncwarp();
#pragma unroll 4
            for (int i = 0; i < 32; ++i) {
                const i64 r = r0 + i;
                if (r < p.n_outer && col < p.len) {
                    VU u;
                    u.vv = *reinterpret_cast<const VV*>(tw + i * RS + lane * VEC);
                    st_out<RT, K_CONTIG, VEC>(reinterpret_cast<RT*>(p.out), r * p.oso + col * p.osa, p.osa, u.e);
                }
            }
            __syncwarp();
        }
    }
}

// K9c: a few long rows (and the flattened form) — segmented
// reduce-then-scan (k_scan_seg_* below), one warp per segment, no warp
// waiting on another.
// ScanState carries float32
// values in double-float (TwoSum for sums, fma-exact TwoProd for products) so
// the tile results are within a few ulp of the exact prefix; other types fold
// in their own arithmetic.  The additive identity is -0 (x + -0 == x for
// every x), so signed zeros come out as in the sequential fold.
template <class RT, int OP> struct ScanState {
    RT hi;
    RT lo;
    static XTG_DI ScanState ident() {
        ScanState s;
        s.hi = (OP & 1) ? RT(1) : (IsFloat<RT>::value ? RT(-0.0) : RT(0));
        s.lo = RT(0);
        return s;
    }
    XTG_DI void add(RT x) {
        if (OP >= 2 && is_nan_v(x)) return;
        if (OP & 1) hi = RT(hi * x);
        else hi = RT(hi + x);
    }
    // partial results combine unconditionally (a NaN partial from inf - inf
    // stays NaN, as the sequential fold's accumulator does)
    XTG_DI void merge(const ScanState& o) {
        if (OP & 1) hi = RT(hi * o.hi);
        else hi = RT(hi + o.hi);
    }
    XTG_DI RT value() const { return hi; }
};
template <int OP> struct ScanState<float, OP> {
    float hi, lo;
    static XTG_DI ScanState ident() {
        ScanState s;
        s.hi = (OP & 1) ? 1.f : -0.f;
        s.lo = 0.f;
        return s;
    }
    XTG_DI void add(float x) {
        if (OP >= 2 && !(x == x)) return;
        if (OP & 1) {
            const float ph = hi * x;
            const float e = fmaf(hi, x, -ph);
            lo = fmaf(lo, x, e);
            hi = ph;
        } else {
            float s, e;
            two_sum(hi, x, s, e);
            hi = s;
            lo += e;
        }
    }
    // (hi, lo) with |lo| <= ulp(hi) / 2 (Fast2Sum; |hi| >= |lo| holds for
    // these states).  add() leaves lo to grow (its rounding errors of hi * x
    // drift one way over long runs, to ~1e-3 of hi after 10^5 products),
    // which is harmless along one chain but not in a product of two states,
    // where lo * o.lo is dropped.  Non-finite states stay as they are.
    static XTG_DI void norm2(float h, float l, float& nh, float& nl) {
        const float s = h + l;
        if (s - s == 0.f) {  // finite
            nh = s;
            nl = l - (s - h);
        } else {
            nh = h;
            nl = l;
        }
    }
    XTG_DI void merge(const ScanState& o) {
        if (OP & 1) {
            float ah, al, bh, bl;
            norm2(hi, lo, ah, al);
            norm2(o.hi, o.lo, bh, bl);
            const float ph = ah * bh;
            const float e = fmaf(ah, bh, -ph);
            lo = fmaf(ah, bl, fmaf(al, bh, e));
            hi = ph;
        } else {
            float s, e;
            two_sum(hi, o.hi, s, e);
            hi = s;
            lo = (lo + o.lo) + e;
        }
    }
    XTG_DI float value() const { return lo == 0.f ? hi : hi + lo; }
};


template <class Tree, class LS, class RT>
XTG_DI RT scan_elem(const ScanParams& p, const Ctx<0>& c, i64 row, i64 k) {
    typedef typename LS::template R<1>::type RG;
    i64 off[XTG_KMAX_LEAVES], inner[XTG_KMAX_LEAVES];
#pragma unroll
    for (int l = 0; l < LS::N; ++l) {
        off[l] = row * p.lso[l] + k * p.lsa[l];
        inner[l] = 0;
    }
    RG rg;
    LoadLeavesAt<LS>::template run<1>(rg, p.leaf, off, inner);
    return cvt<RT>(Tree::ev(rg, 0, c));
}

// In-order block scan of one state per thread (Kogge-Stone inside each warp,
// warp totals in warp order): returns the block total and this thread's
// exclusive prefix.  Fixed structure, so results do not depend on timing.
template <class ST> XTG_DI ST block_inorder_scan(ST v, ST* wsum, ST& excl_in_block) {
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    ST inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        ST y = shfl_up_pod(inc, d);
        if (lane >= d) {
            y.merge(inc);
            inc = y;
        }
    }
    const ST lex = shfl_up_pod(inc, 1);
    __syncthreads();
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    // warp 0 scans the warp totals in order: wsum[w] becomes the exclusive
    // prefix of warp w, wsum[nw] the block total
    const int nw = (int)(blockDim.x >> 5);
    if (warp == 0) {
        ST v2 = lane < nw ? wsum[lane] : ST::ident();
        ST i2 = v2;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            ST y = shfl_up_pod(i2, d);
            if (lane >= d) {
                y.merge(i2);
                i2 = y;
            }
        }
        const ST e2 = shfl_up_pod(i2, 1);
        __syncwarp();
        if (lane < nw) wsum[lane] = lane == 0 ? ST::ident() : e2;
        if (lane == nw - 1) wsum[nw] = i2;
    }
    __syncthreads();
    ST pre = wsum[warp];
    if (lane > 0) pre.merge(lex);
    excl_in_block = pre;
    return wsum[nw];
}

// Segmented reduce-then-scan, one warp per segment (no warp ever waits on
// another, and no block barrier): a row is cut into segments of whole units
// of 512 elements, about one segment per resident warp of the apply pass;
// (A) each segment's total, (B) per row, the exclusive prefixes of the
// segment totals in order, (C) each segment again, warp tile by warp tile
// (32 lanes x IPT consecutive elements per lane), from its prefix: every
// lane folds its IPT elements, the warp scans the lane totals in lane order,
// every lane rescans its elements from (carry, the lanes before it) and the
// tile total joins the carry.  A fixed structure, so results do not depend
// on timing.  With CS (float64 operands streamed by the apply pass) pass A
// also stores every lane's fold of every tile, and pass C takes the lane
// totals from there instead of folding again — the same values, one FP64
// add per element less on a part whose FP64 rate bounds this scan.
// ScanParams.ntiles = units per row; segments per row and units per segment
// ride in n_inner (unused for these rows) as nseg * 2^32 + seg_units.
constexpr int XTG_SCAN_UNIT = 512;
XTG_DI i64 seg_units_of(const ScanParams& p) { return p.n_inner & 0xffffffffll; }
XTG_DI i64 nseg_of(const ScanParams& p) { return p.n_inner >> 32; }

// A lane's IPT consecutive elements into registers: VEC-wide loads when all
// lie before `ke` (VEC > 1: every leaf contiguous or broadcast along the
// row, rows VEC-aligned — the host checks), else one by one.
template <class Tree, class LS, class RT, int VEC, int IPT>
XTG_DI void scan_loadv(const ScanParams& p, const Ctx<0>& c, i64 row, i64 kt, i64 ke, RT (&v)[IPT]) {
    if (VEC > 1 && kt + IPT <= ke) {
        typedef typename LS::template R<VEC>::type RG;
#pragma unroll
        for (int m = 0; m < IPT / VEC; ++m) {
            i64 off[XTG_KMAX_LEAVES];
#pragma unroll
            for (int l = 0; l < LS::N; ++l) off[l] = row * p.lso[l] + (kt + m * VEC) * p.lsa[l];
            RG rg;
            LoadLeavesAt<LS>::template run<VEC>(rg, p.leaf, off, p.lsa);
#pragma unroll
            for (int j = 0; j < VEC; ++j) v[m * VEC + j] = cvt<RT>(Tree::ev(rg, j, c));
        }
    } else {
#pragma unroll
        for (int i = 0; i < IPT; ++i) v[i] = kt + i < ke ? scan_elem<Tree, LS, RT>(p, c, row, kt + i) : RT(0);
    }
}

// VEC == 1 (strided leaves): a warp tile through the warp's own buffer in
// shared memory — coalesced loads (lane l takes l, l + 32, ...), then each
// lane its IPT consecutive elements (rows padded by one element per 32).
template <class Tree, class LS, class RT, int IPT>
XTG_DI void scan_loadw(const ScanParams& p, const Ctx<0>& c, i64 row, i64 k0, i64 ke, RT* wb, RT (&v)[IPT]) {
    const int lane = (int)threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
        const int q = i * 32 + lane;
        if (k0 + q < ke) wb[q + (q >> 5)] = scan_elem<Tree, LS, RT>(p, c, row, k0 + q);
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
        const int q = lane * IPT + i;
        v[i] = k0 + q < ke ? wb[q + (q >> 5)] : RT(0);
    }
    __syncwarp();
}

// The warp tiles [kb, ke) of one row in order, each handed to f(v, k0) in
// the lanes' registers; with VEC > 1 the next tile's loads are in flight
// while f works on the current one.
template <class Tree, class LS, class RT, int VEC, int IPT, class F>
XTG_DI void scan_walk(const ScanParams& p, const Ctx<0>& c, i64 row, i64 kb, i64 ke, RT* wb, F&& f) {
    constexpr int WT = 32 * IPT;
    const i64 lofs = (i64)((int)threadIdx.x & 31) * IPT;
    if constexpr (VEC > 1) {
        RT va[IPT], vb[IPT];
        if (kb < ke) scan_loadv<Tree, LS, RT, VEC, IPT>(p, c, row, kb + lofs, ke, va);
        for (i64 k0 = kb; k0 < ke; k0 += 2 * WT) {
            if (k0 + WT < ke) scan_loadv<Tree, LS, RT, VEC, IPT>(p, c, row, k0 + WT + lofs, ke, vb);
            f(va, k0);
            if (k0 + WT >= ke) break;
            if (k0 + 2 * WT < ke) scan_loadv<Tree, LS, RT, VEC, IPT>(p, c, row, k0 + 2 * WT + lofs, ke, va);
            f(vb, k0 + WT);
        }
    } else {
        RT v[IPT];
        for (i64 k0 = kb; k0 < ke; k0 += WT) {
            scan_loadw<Tree, LS, RT, IPT>(p, c, row, k0, ke, wb, v);
            f(v, k0);
        }
    }
}

// In-order inclusive scan of one state per lane (Kogge-Stone: the earlier
// lanes' part always on the left).
template <class ST> XTG_DI ST warp_inorder_scan(ST v) {
    const int lane = (int)threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        ST y = shfl_up_pod(v, d);
        if (lane >= d) {
            y.merge(v);
            v = y;
        }
    }
    return v;
}

// Shared-memory elements per warp for the VEC == 1 tile buffer.
template <int VEC, int IPT> struct ScanWarpBuf {
    static constexpr int n = VEC > 1 ? 1 : 32 * IPT + IPT;
};

// Lane totals of pass A kept for pass C: one value per (row, warp tile, lane).
template <class RT> XTG_DI RT* scan_csum(const ScanParams& p) {
    return reinterpret_cast<RT*>(reinterpret_cast<char*>(p.agg) + p.csum_off);
}

// A lane's fold of its IPT elements in H independent chains of IPT / H
// consecutive elements (H = 2 for float64: the FP64 results come back
// through a long-latency path, so two chains in flight halve the wait),
// range-checked when the tile ends inside the lane.
template <int H, class ST, class RT, int IPT>
XTG_DI void lane_fold(ST (&h)[H], const RT (&v)[IPT], i64 kt, i64 ke) {
    constexpr int L = IPT / H;
#pragma unroll
    for (int j = 0; j < H; ++j) h[j] = ST::ident();
    if (kt + IPT <= ke) {
#pragma unroll
        for (int i = 0; i < L; ++i)
#pragma unroll
            for (int j = 0; j < H; ++j) h[j].add(v[j * L + i]);
    } else {
#pragma unroll
        for (int i = 0; i < L; ++i)
#pragma unroll
            for (int j = 0; j < H; ++j)
                if (kt + j * L + i < ke) h[j].add(v[j * L + i]);
    }
}

template <class Tree, class LS, class RT, int OP, int VEC, int IPT, bool CS, int H>
__global__ void __launch_bounds__(256) k_scan_seg_reduce(const ScanParams p) {
    pdl_wait();
    typedef ScanState<RT, OP> ST;
    constexpr int WB = ScanWarpBuf<VEC, IPT>::n, WT = 32 * IPT;
    __shared__ RT wbuf[8 * WB];
    Ctx<0> c;
    c.scal = p.scal;
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    RT* wb = wbuf + warp * WB;
    const i64 nseg = nseg_of(p), su = seg_units_of(p);
    const i64 nitems = p.n_outer * nseg;
    const i64 lofs = (i64)lane * IPT;
    const i64 tiles_per_row = p.ntiles * (XTG_SCAN_UNIT / WT);
    for (i64 it = (i64)blockIdx.x * 8 + warp; it < nitems; it += (i64)gridDim.x * 8) {
        const i64 row = it / nseg, sg = it - row * nseg;
        const i64 kb = sg * su * XTG_SCAN_UNIT;
        const i64 ke = kb + su * XTG_SCAN_UNIT < p.len ? kb + su * XTG_SCAN_UNIT : p.len;
        ST s = ST::ident();
        scan_walk<Tree, LS, RT, VEC, IPT>(p, c, row, kb, ke, wb, [&](RT(&v)[IPT], i64 k0) {
            // the lane's fold of each tile (what pass C folds), then merged
            ST hs[H];
            lane_fold<H>(hs, v, k0 + lofs, ke);
            if constexpr (CS) {
                RT* cs = scan_csum<RT>(p) + ((row * tiles_per_row + k0 / WT) * 32 + lane) * H;
#pragma unroll
                for (int j = 0; j < H; ++j) cs[j] = hs[j].hi;
            }
#pragma unroll
            for (int j = 0; j < H; ++j) s.merge(hs[j]);
        });
        const ST tot = warp_inorder_scan(s);
        if (lane == 31) reinterpret_cast<ST*>(p.agg)[it] = tot;
    }
}

// (B) one CTA per row: exclusive prefixes of the row's segment totals, in
// place.  The row's totals (at most one per resident warp: under 160 KB)
// are staged in shared memory by coalesced asynchronous copies, all in
// flight at once; thread t owns the run of
// `per` consecutive totals from t * per: it folds them in order, one block
// scan of the runs' totals gives each run its prefix, and the thread
// rewrites its run from that prefix.
template <class RT, int OP>
__global__ void __launch_bounds__(256) k_scan_seg_offsets(const ScanParams p) {
    pdl_wait();
    typedef ScanState<RT, OP> ST;
    __shared__ ST wsum[9];
    extern __shared__ __align__(16) unsigned char seg_smem[];
    ST* sa = reinterpret_cast<ST*>(seg_smem);
    const i64 nseg = nseg_of(p);
    const i64 per = (nseg + 255) / 256;
    const i64 b0 = (i64)threadIdx.x * per;
    const i64 b1 = b0 + per < nseg ? b0 + per : nseg;
    for (i64 row = blockIdx.x; row < p.n_outer; row += gridDim.x) {
        ST* a = reinterpret_cast<ST*>(p.agg) + row * nseg;
        if constexpr (sizeof(ST) == 16 || sizeof(ST) == 8 || sizeof(ST) == 4) {
            // every copy in flight at once
            for (i64 i = threadIdx.x; i < nseg; i += 256) cp_async<(int)sizeof(ST)>(&sa[i], &a[i]);
            cp_async_commit();
            cp_async_wait<0>();
        } else {
            for (i64 i = threadIdx.x; i < nseg; i += 256) sa[i] = a[i];
        }
        __syncthreads();
        ST run = ST::ident();
        for (i64 i = b0; i < b1; ++i) run.merge(sa[i]);
        ST pre;
        block_inorder_scan(run, wsum, pre);
        for (i64 i = b0; i < b1; ++i) {
            const ST v = sa[i];
            sa[i] = pre;
            pre.merge(v);
        }
        __syncthreads();
        for (i64 i = threadIdx.x; i < nseg; i += 256) a[i] = sa[i];
        __syncthreads();
    }
}

// (C) each segment again from its prefix.  Results leave the lanes'
// registers: 16-byte stores when the lane's elements are whole (VEC > 1:
// the destination contiguous and aligned — the host checks).  NS > 0 (the
// operand a plain contiguous array of the accumulation type, 4 or 8 bytes,
// rows 16-byte aligned): every lane streams its own 16-byte chunks of the
// next NS - 1 tiles into a per-warp ring in shared memory with cp.async, so
// tiles are in flight without holding registers; a lane reads back only
// what it copied itself (visible to it after cp.async.wait_group), so no
// barrier is involved.  Chunk m of a lane lands in slot (m + rot) mod CPL of
// the lane's 16-byte slots, rot = the lane's position within its 128 bytes
// of the stage: the lanes of one 8-lane phase of a 16-byte read hit
// distinct banks.  Four blocks per SM for 4-byte types with vector access
// (a register bound of 64, no spill), fewer otherwise.
template <class Tree, class LS, class RT, int OP, int VEC, int NS, int IPT, bool CS, int H>
__global__ void __launch_bounds__(256, VEC > 1 && sizeof(RT) <= 4 ? 4 : NS > 0 && IPT <= 8 ? 3 : 2)
    k_scan_seg_apply(const ScanParams p) {
    pdl_wait();
    typedef ScanState<RT, OP> ST;
    constexpr int WB = NS > 0 ? 1 : ScanWarpBuf<VEC, IPT>::n, WT = 32 * IPT;
    __shared__ RT wbuf[8 * WB];
    extern __shared__ __align__(16) unsigned char ring[];
    Ctx<0> c;
    c.scal = p.scal;
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    RT* wb = wbuf + warp * WB;
    const i64 nseg = nseg_of(p), su = seg_units_of(p);
    const i64 nitems = p.n_outer * nseg;
    const i64 lofs = (i64)lane * IPT;
    const i64 tiles_per_row = p.ntiles * (XTG_SCAN_UNIT / WT);
    for (i64 it = (i64)blockIdx.x * 8 + warp; it < nitems; it += (i64)gridDim.x * 8) {
        const i64 row = it / nseg, sg = it - row * nseg;
        const i64 kb = sg * su * XTG_SCAN_UNIT;
        const i64 ke = kb + su * XTG_SCAN_UNIT < p.len ? kb + su * XTG_SCAN_UNIT : p.len;
        ST carry = reinterpret_cast<const ST*>(p.agg)[it];
        RT* o = reinterpret_cast<RT*>(p.out) + row * p.oso;
        auto tile = [&](RT(&v)[IPT], i64 k0, const RT* csv) {
            const i64 kt = k0 + lofs;
            // every tile but a row's last is whole: no per-element checks
            const bool full = kt + IPT <= ke;
            ST hs[H];
            if constexpr (CS) {
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    hs[j] = ST::ident();
                    hs[j].hi = csv[j];
                }
            } else {
                lane_fold<H>(hs, v, kt, ke);
            }
            ST s = ST::ident();
#pragma unroll
            for (int j = 0; j < H; ++j) s.merge(hs[j]);
            const ST inc = warp_inorder_scan(s);
            const ST lex = shfl_up_pod(inc, 1);
            const ST tile_tot = shfl_idx_pod(inc, 31);
            ST pre = carry;
            if (lane > 0) pre.merge(lex);
            if (full && kt != 0) {
                // chain j starts from the prefix plus the folds before it
                constexpr int L = IPT / H;
                ST pr[H];
                pr[0] = pre;
#pragma unroll
                for (int j = 1; j < H; ++j) {
                    pr[j] = pr[j - 1];
                    pr[j].merge(hs[j - 1]);
                }
#pragma unroll
                for (int i = 0; i < L; ++i)
#pragma unroll
                    for (int j = 0; j < H; ++j) {
                        pr[j].add(v[j * L + i]);
                        v[j * L + i] = pr[j].value();
                    }
            } else {
#pragma unroll
                for (int i = 0; i < IPT; ++i) {
                    const i64 k = kt + i;
                    if (k < ke) {
                        if (k == 0) {
                            pre.hi = ScanOp<RT, OP>::init(v[i]);
                            pre.lo = RT(0);
                        } else {
                            pre.add(v[i]);
                        }
                        v[i] = pre.value();
                    }
                }
            }
            if (VEC > 1 && full) {
#pragma unroll
                for (int m = 0; m < IPT / VEC; ++m) {
                    RT w[VEC > 1 ? VEC : 1];
#pragma unroll
                    for (int j = 0; j < VEC; ++j) w[j] = v[m * VEC + j];
                    st_out<RT, K_CONTIG, VEC>(o, kt + m * VEC, 1, w);
                }
            } else {
#pragma unroll
                for (int i = 0; i < IPT; ++i)
                    if (kt + i < ke) o[(kt + i) * p.osa] = v[i];
            }
            carry.merge(tile_tot);
        };
        if constexpr (NS > 0) {
            constexpr int EPC = 16 / (int)sizeof(RT);        // elements per 16-byte chunk
            constexpr int CPL = IPT / EPC;                   // chunks per lane
            constexpr int SB = 32 * IPT * (int)sizeof(RT);   // bytes of a warp tile
            // a stage: the warp tile, then (CS) the 32 lanes' H folds from pass A
            constexpr int CSB = H * (int)sizeof(RT);
            constexpr int SBX = SB + (CS ? 32 * CSB : 0);
            unsigned char* wbase = ring + (size_t)warp * NS * SBX;
            unsigned char* wr = wbase + (size_t)lane * CPL * 16;
            const int rot = (lane / (CPL >= 8 ? 1 : 8 / CPL)) % CPL;
            const RT* src = reinterpret_cast<const RT*>(p.leaf[0]) + row * p.lso[0];
            const i64 T = (ke - kb + WT - 1) / WT;
            auto issue = [&](i64 t) {
                const i64 kt = kb + t * WT + lofs;
                if (t < T && kt + IPT <= ke) {
                    unsigned char* d = wr + (int)(t % NS) * SBX;
#pragma unroll
                    for (int m = 0; m < CPL; ++m) cp_async<16>(d + ((m + rot) % CPL) * 16, src + kt + m * EPC);
                }
                if (CS && t < T)
                    cp_async<CSB>(wbase + (int)(t % NS) * SBX + SB + lane * CSB,
                                  scan_csum<RT>(p) + ((row * tiles_per_row + (kb + t * WT) / WT) * 32 + lane) * H);
                cp_async_commit();
            };
#pragma unroll 1
            for (int j = 0; j < NS - 1; ++j) issue(j);
            for (i64 t = 0; t < T; ++t) {
                // the slot of tile t + NS - 1 was read back (into registers
                // already used) while tile t - 1 was scanned
                issue(t + NS - 1);
                cp_async_wait<NS - 1>();
                const i64 k0 = kb + t * WT, kt = k0 + lofs;
                RT csv[H];
#pragma unroll
                for (int j = 0; j < H; ++j)
                    csv[j] = CS ? reinterpret_cast<const RT*>(wbase + (int)(t % NS) * SBX + SB + lane * CSB)[j] : RT(0);
                RT v[IPT];
                if (kt + IPT <= ke) {
                    const unsigned char* d = wr + (int)(t % NS) * SBX;
#pragma unroll
                    for (int m = 0; m < CPL; ++m) {
                        union {
                            uint4 q;
                            RT e[EPC];
                        } u;
                        u.q = *reinterpret_cast<const uint4*>(d + ((m + rot) % CPL) * 16);
#pragma unroll
                        for (int j = 0; j < EPC; ++j) v[m * EPC + j] = u.e[j];
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < IPT; ++i) v[i] = kt + i < ke ? src[kt + i] : RT(0);
                }
                tile(v, k0, csv);
            }
        } else {
            static_assert(!CS, "lane totals from pass A come with the streamed form");
            scan_walk<Tree, LS, RT, VEC, IPT>(p, c, row, kb, ke, wb,
                                              [&](RT(&v)[IPT], i64 k0) { tile(v, k0, nullptr); });
        }
    }
}

// ---------------------------------------------------------------------------
// K10: indexed evaluation — reads and writes through xt::index_view, filter
// and filtration (include/xtensor/views/xindex_view.hpp:54-206, 786-850).
// VT: value type of the evaluated tree; DT: destination type; CT: the type
// `dst op value` computes in (C++ conversions); OP: xtg_set_op.  MODE 0:
// out[k] = e[idx[k]] (gather), MODE 1: dst[idx[k]] op= src[k] (scatter).
// 2^24 random 4-byte accesses run at about 40 G/s, the rate of random
// 32-byte sectors on HBM3e; more coordinates in flight per thread did not
// raise it.
template <class Tree, class LS, class VT, class DT, class CT, int MODE, int R, int OP>
__global__ void __launch_bounds__(256) k_indexed(const IndexParams p) {
    pdl_wait();
    typedef typename LS::template R<1>::type RG;
    Ctx<0> c;
    c.scal = p.scal;
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < p.n; k += (i64)gridDim.x * blockDim.x) {
        i64 ix[R > 0 ? R : 1];
        i64 j = 0;  // 1-D position in the out (mode 0) or src (mode 1) space
        {
            bool ok = true;
#pragma unroll
            for (int d = 0; d < R; ++d) {
                ix[d] = p.idx[k * R + d];
                if (ix[d] < 0 || ix[d] >= p.shape[d]) ok = false;
            }
            if (!ok) {
                atomicExch(p.err, 2);  // reported as XTG_ERR_OUT_OF_RANGE
                continue;
            }
            j = k;
        }
        i64 off[XTG_KMAX_LEAVES], inner[XTG_KMAX_LEAVES];
#pragma unroll
        for (int l = 0; l < LS::N; ++l) {
            inner[l] = 0;
            if (MODE == 0) {
                i64 o = 0;
#pragma unroll
                for (int d = 0; d < R; ++d) o += ix[d] * p.ls[l][d];
                off[l] = o;
            } else {
                off[l] = j * p.ls[l][0];
            }
        }
        RG rg;
        LoadLeavesAt<LS>::template run<1>(rg, p.leaf, off, inner);
        const VT v = cvt<VT>(Tree::ev(rg, 0, c));
        DT* dst = reinterpret_cast<DT*>(p.dst);
        if (MODE == 0) {
            dst[j * p.ds[0]] = cvt<DT>(v);
        } else {
            i64 o = 0;
#pragma unroll
            for (int d = 0; d < R; ++d) o += ix[d] * p.ds[d];
            if (OP == 0) {
                dst[o] = cvt<DT>(v);
            } else {
                const CT a = cvt<CT>(dst[o]), b = cvt<CT>(v);
                const CT r = OP == 1 ? CT(a + b) : OP == 2 ? CT(a - b) : OP == 3 ? CT(a * b) : CT(a / b);
                dst[o] = cvt<DT>(r);
            }
        }
    }
}

// K11: filters — xt::filter(e, cond) reads and filter / filtration writes
// (include/xtensor/views/xindex_view.hpp:786-850).  Thread th of a tile owns
// the 16 consecutive positions t*4096 + 16 th .. + 15, so the selected
// elements come out in row-major order: (A) count per tile, (B) an
// inclusive scan of the counts (the accumulator kernels), (C) every tile
// again, each selected element to tile offset + its rank in the tile.
template <class Tree, class LS, int R, bool BIG>
XTG_DI bool filter_cond(const FilterParams& p, const Ctx<0>& c, i64 k, i64 (&ix)[R]) {
    typedef typename LS::template R<1>::type RG;
    decode_dims<R, BIG>(p.shape, p.fd, k, ix);
    i64 off[XTG_KMAX_LEAVES], inner[XTG_KMAX_LEAVES];
#pragma unroll
    for (int l = 0; l < LS::N; ++l) {
        i64 o = 0;
#pragma unroll
        for (int d = 0; d < R; ++d) o += ix[d] * p.cls[l][d];
        off[l] = o;
        inner[l] = 0;
    }
    RG rg;
    LoadLeavesAt<LS>::template run<1>(rg, p.cleaf, off, inner);
    return Tree::ev(rg, 0, c) != typename Tree::type(0);
}

// One flat dim (R == 1), every condition leaf contiguous (stride 1, 16-byte
// aligned) or broadcast (stride 0): the 16 consecutive positions of a
// thread are read with 16-byte loads.
template <int I, class... S> struct LoadFlat16;
template <int I> struct LoadFlat16<I> {
    template <class RG> static XTG_DI void run(RG&, const void* const*, i64, const i64 (*)[XTG_KMAX_RANK]) {}
};
template <int I, class S0, class... S> struct LoadFlat16<I, S0, S...> {
    template <class RG> static XTG_DI void run(RG& rg, const void* const* ptr, i64 k0, const i64 (*st)[XTG_KMAX_RANK]) {
        typedef typename S0::type T;
        const T* b = reinterpret_cast<const T*>(ptr[I]);
        if (st[I][0] != 0) {
            constexpr int NV = (int)sizeof(T) * 16 / 16;  // 16-byte vectors for 16 elements
            union { uint4 v[NV]; T e[16]; } u;
#pragma unroll
            for (int q = 0; q < NV; ++q) u.v[q] = __ldg(reinterpret_cast<const uint4*>(b + k0) + q);
#pragma unroll
            for (int j = 0; j < 16; ++j) rg.v[j] = u.e[j];
        } else {
            const T v = ld1<T>(b);
#pragma unroll
            for (int j = 0; j < 16; ++j) rg.v[j] = v;
        }
        LoadFlat16<I + 1, S...>::run(rg.rest, ptr, k0, st);
    }
};
template <class LS> struct CondFlat16;
template <class... S> struct CondFlat16<LeafSet<S...>> {
    template <class Tree> static XTG_DI unsigned run(const FilterParams& p, const Ctx<0>& c, i64 k0) {
        typename LeafSet<S...>::template R<16>::type rg;
        LoadFlat16<0, S...>::run(rg, p.cleaf, k0, p.cls);
        unsigned f = 0;
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (Tree::ev(rg, j, c) != typename Tree::type(0)) f |= 1u << j;
        return f;
    }
};
// The condition flags of positions k0 .. k0 + 15 (bit i: position k0 + i).
template <class CTree, class CLS, int R, bool BIG, bool V16>
XTG_DI unsigned filter_flags16(const FilterParams& p, const Ctx<0>& c, i64 k0) {
    if (V16 && k0 + 16 <= p.n) return CondFlat16<CLS>::template run<CTree>(p, c, k0);
    unsigned flags = 0;
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
        const i64 k = k0 + i;
        i64 ix[R];
        if (k < p.n && filter_cond<CTree, CLS, R, BIG>(p, c, k, ix)) flags |= 1u << i;
    }
    return flags;
}

template <class CTree, class CLS, int R, bool BIG, bool V16 = false>
__global__ void __launch_bounds__(256) k_filter_count(const FilterParams p) {
    pdl_wait();
    __shared__ int ws[8];
    Ctx<0> c;
    c.scal = p.cscal;
    const i64 ntiles = (p.n + 4095) / 4096;
    for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const i64 k0 = t * 4096 + (i64)threadIdx.x * 16;
        int cnt = __popc(filter_flags16<CTree, CLS, R, BIG, V16>(p, c, k0));
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0;
            for (int w = 0; w < 8; ++w) s += ws[w];
            p.tcount[t] = s;
        }
        __syncthreads();
    }
}

// MODE 0: out[j] = e[position]; MODE 1: dst[position] = dst op src[j]
template <class CTree, class CLS, class VTree, class VLS, class VT, class DT, class CT, int MODE, int R, int OP, bool BIG,
          bool V16 = false>
__global__ void __launch_bounds__(256) k_filter_tile(const FilterParams p) {
    pdl_wait();
    typedef typename VLS::template R<1>::type VRG;
    __shared__ int ws[9];
    Ctx<0> cc, vc;
    cc.scal = p.cscal;
    vc.scal = p.vscal;
    const i64 ntiles = (p.n + 4095) / 4096;
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const i64 k0 = t * 4096 + (i64)threadIdx.x * 16;
        unsigned flags = filter_flags16<CTree, CLS, R, BIG, V16>(p, cc, k0);
        // exclusive prefix of the thread counts in thread order
        const int cnt = __popc(flags);
        int inc = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += y;
        }
        if (lane == 31) ws[warp] = inc;
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0;
            for (int w = 0; w < 8; ++w) {
                const int v = ws[w];
                ws[w] = s;
                s += v;
            }
        }
        __syncthreads();
        i64 j = (t ? (i64)p.tincl[t - 1] : 0) + ws[warp] + (inc - cnt);
        while (flags) {
            const int i = __ffs(flags) - 1;
            flags &= flags - 1;
            const i64 k = k0 + i;
            i64 ix[R];
            decode_dims<R, BIG>(p.shape, p.fd, k, ix);
            i64 off[XTG_KMAX_LEAVES], inner[XTG_KMAX_LEAVES];
#pragma unroll
            for (int l = 0; l < VLS::N; ++l) {
                inner[l] = 0;
                if (MODE == 0) {
                    i64 o = 0;
#pragma unroll
                    for (int d = 0; d < R; ++d) o += ix[d] * p.vls[l][d];
                    off[l] = o;
                } else {
                    off[l] = j * p.vls[l][0];
                }
            }
            VRG rg;
            LoadLeavesAt<VLS>::template run<1>(rg, p.vleaf, off, inner);
            const VT v = cvt<VT>(VTree::ev(rg, 0, vc));
            DT* dst = reinterpret_cast<DT*>(p.dst);
            if (MODE == 0) {
                dst[j * p.ds[0]] = cvt<DT>(v);
            } else {
                i64 o = 0;
#pragma unroll
                for (int d = 0; d < R; ++d) o += ix[d] * p.ds[d];
                if (OP == 0) {
                    dst[o] = cvt<DT>(v);
                } else {
                    const CT a = cvt<CT>(dst[o]), b = cvt<CT>(v);
                    const CT r = OP == 1 ? CT(a + b) : OP == 2 ? CT(a - b) : OP == 3 ? CT(a * b) : CT(a / b);
                    dst[o] = cvt<DT>(r);
                }
            }
            ++j;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// K2: tiled transposing assignment (transpose / permuted strided_view into a
// contiguous destination — the case xtensor sends to the scalar
// stepper_assigner, include/xtensor/core/xassign.hpp:1087, 1341).
// Dims are in destination order after collapsing; dim B = R-1 is contiguous
// in the destination, dim A (p.da) is the one along which leaf 0 — the
// transposed source — is unit-stride.  A TILE x TILE tile goes through shared
// memory: loads walk A (coalesced for leaf 0), stores walk B (coalesced for
// the destination).  Other leaves are read directly at (a, b).
template <class Tree, class LS, class OutT, int NB, int TILE, int ROWS>
__global__ void __launch_bounds__(TILE * ROWS) k_transpose(const TransposeParams p) {
    pdl_wait();
    typedef typename LS::template R<1>::type RG;
    typedef typename RG::elem0 T0;
    __shared__ T0 tile[TILE][TILE + 1];
    Ctx<0> c;
    c.scal = p.scal;
    const int tx = threadIdx.x % TILE, ty = threadIdx.x / TILE;
    for (i64 t = blockIdx.x; t < p.n_tiles; t += gridDim.x) {
        i64 tb = t % p.ntile_b;
        i64 rest = t / p.ntile_b;
        i64 ta = rest % p.ntile_a;
        i64 bt = rest / p.ntile_a;
        i64 boff[XTG_KMAX_LEAVES];
        i64 obo = 0;
#pragma unroll
        for (int l = 0; l < LS::N; ++l) boff[l] = 0;
#pragma unroll
        for (int d = NB - 1; d >= 0; --d) {
            i64 n = p.bshape[d];
            i64 q = bt / n;
            i64 id = bt - q * n;
            bt = q;
            obo += id * p.obs[d];
#pragma unroll
            for (int l = 0; l < LS::N; ++l) boff[l] += id * p.lbs[l][d];
        }
        const i64 a0 = ta * TILE, b0 = tb * TILE;
        const T0* src = reinterpret_cast<const T0*>(p.leaf[0]);
        if (LS::N == 1 && a0 + TILE <= p.sa && b0 + TILE <= p.sb) {
            // interior tile of a single-leaf tree: no bounds tests, and one
            // pointer step per element instead of the 64-bit index products
            const T0* ps = src + boff[0] + (a0 + tx) * p.la[0] + (b0 + ty) * p.lb[0];
            const i64 sstep = (i64)ROWS * p.lb[0];
#pragma unroll
            for (int bb = ty; bb < TILE; bb += ROWS) {
                tile[bb][tx] = ld1<T0>(ps);
                ps += sstep;
            }
            __syncthreads();
            OutT* pd = reinterpret_cast<OutT*>(p.out) + obo + (a0 + ty) * p.oa + (b0 + tx) * p.ob;
            const i64 dstep = (i64)ROWS * p.oa;
#pragma unroll
            for (int aa = ty; aa < TILE; aa += ROWS) {
                RG rg;
                rg.v[0] = tile[tx][aa];
                *pd = cvt<OutT>(Tree::ev(rg, 0, c));
                pd += dstep;
            }
            __syncthreads();
            continue;
        }
        {
            const i64 a = a0 + tx;
#pragma unroll
            for (int bb = ty; bb < TILE; bb += ROWS) {
                const i64 b = b0 + bb;
                if (a < p.sa && b < p.sb) tile[bb][tx] = ld1<T0>(src + boff[0] + a * p.la[0] + b * p.lb[0]);
            }
        }
        __syncthreads();
        {
            const i64 b = b0 + tx;
#pragma unroll
            for (int aa = ty; aa < TILE; aa += ROWS) {
                const i64 a = a0 + aa;
                if (a < p.sa && b < p.sb) {
                    RG rg;
                    rg.v[0] = tile[tx][aa];
                    i64 off[XTG_KMAX_LEAVES], inner[XTG_KMAX_LEAVES];
#pragma unroll
                    for (int l = 0; l < LS::N; ++l) { off[l] = boff[l] + a * p.la[l] + b * p.lb[l]; inner[l] = 0; }
                    LoadRest<LS>::run(rg, p.leaf, off, inner);
                    reinterpret_cast<OutT*>(p.out)[obo + a * p.oa + b * p.ob] = cvt<OutT>(Tree::ev(rg, 0, c));
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// K7: fused row statistics.  Trees holding keep-dims reductions over the
// trailing axes — C1's (x - mean(x,{2},kd)) / sqrt(variance(x,{2},kd) + eps),
// which the reference evaluates with three passes and a temporary
// (include/xtensor/core/xmath.hpp:2082-2103) — run as ONE pass: a group
// (warp or CTA) loads a whole row into registers, computes every statistic
// from registers (two-pass mean / sum of squared deviations, compensated),
// then evaluates the tree and stores the row.  HBM traffic: one read, one
// write.
// A statistic: MODE 0 sum, 1 mean, 2 variance, 3 stddev, 4 max, 5 min;
// C = compute type (float: compensated double-float; double: FP64); Sub is
// the subtree it reduces.
template <int K, int MODE, class C, class Sub> struct RStat {};
template <class... X> struct StatList {};

struct DSum {
    double s;
    XTG_DI void merge(const DSum& o) { s += o.s; }
};
// Row sums: FP64 for float64 (and integer) data, double-float for float32.
template <int GROUP, class C> struct RowSum {
    typedef DSum A;
    static XTG_DI void zero(A& a) { a.s = 0.0; }
    template <class X> static XTG_DI void add(A& a, X v) { a.s += cvt<double>(v); }
    template <class X> static XTG_DI void addsq(A& a, X d) {
        double x = cvt<double>(d);
        a.s = fma(x, x, a.s);
    }
    static XTG_DI double val(const A& a) { return a.s; }
};
template <int GROUP> struct RowSum<GROUP, float> {
    typedef AccSumC A;
    static XTG_DI void zero(A& a) { a.hi = 0.f; a.lo = 0.f; }
    static XTG_DI void add(A& a, float v) { a.addf(v); }
    static XTG_DI void addsq(A& a, float d) {
        float q = d * d;
        float qe = fmaf(d, d, -q);
        a.addf(q);
        a.lo += qe;
    }
    static XTG_DI double val(const A& a) { return a.dval(); }
};
// After group_reduce every lane of a warp group already holds the total: the
// xor butterfly merges the same operands in every lane, and every merge is
// symmetric (sums, exact TwoSum errors, selection with position ties), so a
// warp group needs no broadcast.
template <int GROUP, class A> XTG_DI A bcast_group(A a, A* smem) {
    if (GROUP <= 32) return a;
    __syncthreads();
    if (threadIdx.x == 0) smem[0] = a;
    __syncthreads();
    A r = smem[0];
    return r;
}

// Per-row finalisation of the fused statistics in the row's precision.
template <class C> struct RowFin {  // float64 (and integer) rows: FP64
    template <class A> static XTG_DI double total(const A& a) { return a.s; }
    static XTG_DI double scale(double v, const RowParams& p, int k) { return v * p.rdiv[k]; }
    static XTG_DI double mean(double sum, const RowParams& p) { return sum * p.rrow_len; }
    template <class CT> static XTG_DI void put(CT& c, int k, double v) {
        c.stat[k] = v;
        c.statf[k] = (float)v;
    }
};
template <> struct RowFin<float> {  // float32 rows: double-float sums rounded once, FP32 after
    static XTG_DI float total(const AccSumC& a) { return a.hi + a.lo; }
    static XTG_DI float scale(float v, const RowParams& p, int k) { return v / p.fdiv[k]; }
    static XTG_DI float mean(float sum, const RowParams& p) { return sum / p.frow_len; }
    template <class CT> static XTG_DI void put(CT& c, int k, float v) {
        c.statf[k] = v;
        c.stat[k] = (double)v;
    }
};

// float64 row moments on the integer pipes.  GB300 issues FP64 at a small
// fraction of its FP32 rate, so sum / mean / variance of a float64 row are
// computed in fixed point instead.  With Ef the largest exponent field in
// the row, every element becomes the integer
//   X = round(x * 2^(1075 - Ef)),   |X| < 2^53,
// which is exact for the elements in the top binade; smaller ones are
// rounded to the top binade's ulp (so a row sum is within n/2 of that ulp
// plus one final rounding).  From there on everything is exact:  Each lane (at most 256 elements)
// keeps sum X and sum X^2 exactly in 64-bit words (|X| = Xh * 2^27 + Xl, so
// X^2 = Xh^2 2^54 + 2 Xh Xl 2^27 + Xl^2 as three sums of unsigned 32x32-bit
// products); lanes combine in 128-bit, and
//   n * sum (X - mean)^2 = n * sum X^2 - (sum X)^2
// is evaluated in 192-bit integers, so no cancellation can occur whatever the
// mean.  Rows holding an infinity or NaN take the FP64 path.
struct IMaxI {
    int v;
    XTG_DI void merge(const IMaxI& o) { v = v > o.v ? v : o.v; }
};
struct U128 {
    u64 lo, hi;
};
struct U192 {
    u64 w0, w1, w2;
};
XTG_DI U128 u128_shl(u64 v, int n) {  // v * 2^n, 0 < n < 64
    U128 r;
    r.lo = v << n;
    r.hi = v >> (64 - n);
    return r;
}
XTG_DI U128 u128_add(U128 a, U128 b) {
    U128 r;
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
    return r;
}
XTG_DI U128 u128_sub(U128 a, U128 b) {
    U128 r;
    r.lo = a.lo - b.lo;
    r.hi = a.hi - b.hi - (a.lo < b.lo ? 1ull : 0ull);
    return r;
}
XTG_DI U192 u192_mul(U128 a, u64 m) {  // a * m
    U192 r;
    r.w0 = a.lo * m;
    const u64 c0 = __umul64hi(a.lo, m);
    const u64 p1 = a.hi * m;
    r.w1 = c0 + p1;
    r.w2 = __umul64hi(a.hi, m) + (r.w1 < c0 ? 1ull : 0ull);
    return r;
}
XTG_DI U192 u192_add(U192 a, U192 b) {
    U192 r;
    r.w0 = a.w0 + b.w0;
    const u64 c0 = r.w0 < a.w0 ? 1ull : 0ull;
    const u64 t = a.w1 + b.w1;
    const u64 c1 = t < a.w1 ? 1ull : 0ull;
    r.w1 = t + c0;
    r.w2 = a.w2 + b.w2 + c1 + (r.w1 < t ? 1ull : 0ull);
    return r;
}
XTG_DI U192 u192_sub(U192 a, U192 b) {
    U192 r;
    r.w0 = a.w0 - b.w0;
    const u64 b0 = a.w0 < b.w0 ? 1ull : 0ull;
    const u64 t = a.w1 - b.w1;
    const u64 b1 = a.w1 < b.w1 ? 1ull : 0ull;
    r.w1 = t - b0;
    r.w2 = a.w2 - b.w2 - b1 - (t < b0 ? 1ull : 0ull);
    return r;
}
// (-1)^neg * q * 2^e2 rounded to nearest even, on the integer pipes (a lane
// of a warp group runs this per row, and GB300's FP64 rate makes the usual
// conversions + scalbn cost more than the row's elements).  One rounding in
// every range: results below the normal range round the 64-bit window
// directly to the subnormal grid, results above it are infinities.
XTG_DI double fix_to_double(U192 q, bool neg, int e2) {
    int top;
    if (q.w2) top = 191 - __clzll(q.w2);
    else if (q.w1) top = 127 - __clzll(q.w1);
    else if (q.w0) top = 63 - __clzll(q.w0);
    else return neg ? -0.0 : 0.0;
    // the 64 bits below and including the top bit, and whether anything
    // nonzero lies under them
    u64 m;
    bool sticky;
    const int sh = top - 63;
    if (sh <= 0) {
        m = q.w0 << (-sh);
        sticky = false;
    } else {
        const int wi = sh >> 6, b = sh & 63;
        const u64 lo = wi == 0 ? q.w0 : (wi == 1 ? q.w1 : q.w2);
        const u64 hi = wi == 0 ? q.w1 : (wi == 1 ? q.w2 : 0ull);
        m = b ? ((lo >> b) | (hi << (64 - b))) : lo;
        const u64 below = b ? (lo << (64 - b)) : 0ull;
        sticky = below != 0 || (wi >= 1 && q.w0 != 0) || (wi == 2 && q.w1 != 0);
    }
    if (top + e2 + 1023 < 1) {
        // below the normal range: round the window (and what lies under it)
        // once, straight to the subnormal grid of 2^-1074; a carry into
        // 2^52 is the smallest normal number's bit pattern
        const int r = -(top - 63 + e2 + 1074);  // bits of the window to drop, >= 12
        u64 qv;
        bool rb, st;
        if (r >= 65) {
            qv = 0;
            rb = false;
            st = true;
        } else if (r == 64) {
            qv = 0;
            rb = (m >> 63) & 1;
            st = sticky || (m << 1) != 0;
        } else {
            qv = m >> r;
            rb = (m >> (r - 1)) & 1;
            st = sticky || (m << (65 - r)) != 0;
        }
        if (rb && (st || (qv & 1))) ++qv;
        return __longlong_as_double((long long)(((u64)neg << 63) | qv));
    }
    u64 mant = m >> 11;  // 53 bits, leading one at bit 52
    const bool rnd = (m >> 10) & 1;
    sticky = sticky || (m & 0x3ffull) != 0;
    if (rnd && (sticky || (mant & 1))) ++mant;
    int e = top + e2;  // value = mant * 2^(e - 52)
    if (mant >> 53) {
        mant >>= 1;
        ++e;
    }
    const int be = e + 1023;
    if (be > 2046) return neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
    const u64 bits = ((u64)neg << 63) | ((u64)be << 52) | (mant & 0xfffffffffffffull);
    return __longlong_as_double((long long)bits);
}

// lane / group partial sums: sum X as a signed 128-bit (two's complement)
// word pair, sum X^2 as unsigned 128-bit
struct FixMom {
    U128 s1, s2;
    XTG_DI void merge(const FixMom& o) {
        s1 = u128_add(s1, o.s1);
        s2 = u128_add(s2, o.s2);
    }
};
// |X| for the element with words (hi, lo): twice the significand (< 2^54),
// shifted down to the row's scale, then one add and one shift round it half
// away from zero.  The sign is the sign bit of hi.
XTG_DI u64 fixed_mag(int hi, unsigned lo, int ef_max) {
    const int e = (hi >> 20) & 0x7ff;
    const u64 m2 = (((u64)(unsigned)((hi & 0xfffff) | (e ? 0x100000 : 0)) << 32) | lo) << 1;
    int sh = ef_max - (e ? e : 1);  // subnormals scale like exponent field 1
    sh = sh < 63 ? sh : 63;
    return ((m2 >> sh) + 1) >> 1;
}

template <int GROUP, int VEC, int NV, int MODE, class Sub, class RG, class CT>
XTG_DI bool fixed_moments(const RG (&rg)[NV], const bool (&ok)[NV][VEC], const CT& c, const RowParams& p, void* smem,
                          double& sum, double& sdev2) {
    static_assert(NV * VEC <= 256, "per-lane 64-bit sums hold at most 256 elements");
    const i64 n = p.row_len;
    // the largest exponent field: the high words with the sign cleared order
    // like their exponent fields
    unsigned mh = 0;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int j = 0; j < VEC; ++j)
            if (ok[i][j]) {
                const unsigned h = (unsigned)__double2hiint(cvt<double>(Sub::ev(rg[i], j, c))) & 0x7fffffffu;
                mh = mh > h ? mh : h;
            }
    IMaxI em;
    em.v = (int)(mh >> 20);
    em.v = em.v > 1 ? em.v : 1;
    em = group_reduce<GROUP>(em, reinterpret_cast<IMaxI*>(smem));
    em = bcast_group<GROUP>(em, reinterpret_cast<IMaxI*>(smem));
    if (em.v >= 0x7ff || n > 65536) return false;
    i64 s1 = 0;
    u64 a = 0, b = 0, cc = 0;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int j = 0; j < VEC; ++j)
            if (ok[i][j]) {
                const double xd = cvt<double>(Sub::ev(rg[i], j, c));
                const int hi = __double2hiint(xd);
                const u64 v = fixed_mag(hi, (unsigned)__double2loint(xd), em.v);  // |X| < 2^53
                if (hi < 0) s1 -= (i64)v;
                else s1 += (i64)v;
                if (MODE >= 2) {
                    const unsigned xh = (unsigned)(v >> 27);   // < 2^26
                    const unsigned xl = (unsigned)v & 0x7ffffffu;  // < 2^27
                    a += (u64)xh * xh;
                    b += (u64)xh * xl;
                    cc += (u64)xl * xl;
                }
            }
    FixMom f;
    f.s1.lo = (u64)s1;
    f.s1.hi = s1 < 0 ? ~0ull : 0ull;
    f.s2.lo = 0;
    f.s2.hi = 0;
    if (MODE >= 2) {
        // lane sum X^2 = a 2^54 + b 2^28 + cc  (< 2^116)
        U128 t = u128_shl(a, 54);
        t = u128_add(t, u128_shl(b, 28));
        U128 ct;
        ct.lo = cc;
        ct.hi = 0;
        f.s2 = u128_add(t, ct);
    }
    f = group_reduce<GROUP>(f, reinterpret_cast<FixMom*>(smem));
    f = bcast_group<GROUP>(f, reinterpret_cast<FixMom*>(smem));
    const int sig = em.v - 1075;  // x = X * 2^sig
    U128 m1 = f.s1;
    const bool neg = (i64)m1.hi < 0;
    if (neg) {
        U128 z;
        z.lo = 0;
        z.hi = 0;
        m1 = u128_sub(z, m1);
    }
    U192 s1w;
    s1w.w0 = m1.lo;
    s1w.w1 = m1.hi;
    s1w.w2 = 0;
    sum = fix_to_double(s1w, neg, sig);
    sdev2 = 0.0;
    if (MODE >= 2) {
        // sum X^2 < 2^122, n <= 2^16: n * sum X^2 - (sum X)^2 in 192 bits
        // (exact, >= 0); returned as n * sum (x - mean)^2
        U192 sq = u192_mul(m1, m1.lo);
        const U192 sqh = u192_mul(m1, m1.hi);  // times 2^64
        U192 sh;
        sh.w0 = 0;
        sh.w1 = sqh.w0;
        sh.w2 = sqh.w1;
        sq = u192_add(sq, sh);
        const U192 q = u192_sub(u192_mul(f.s2, (u64)n), sq);
        sdev2 = fix_to_double(q, false, 2 * sig);
    }
    return true;
}

template <class A, class B> struct SameT { enum { value = 0 }; };
template <class A> struct SameT<A, A> { enum { value = 1 }; };
// Statistics of the same float64 operand share one pass of fixed_moments:
// the highest moment any of them needs, and who receives the results.
template <class Sub, class... R> struct SameSubMode { enum { value = -1 }; };
template <class Sub, int K2, int M2, class C2, class S2, class... R> struct SameSubMode<Sub, RStat<K2, M2, C2, S2>, R...> {
    enum {
        rest = SameSubMode<Sub, R...>::value,
        mine = (SameT<Sub, S2>::value && sizeof(C2) == 8 && M2 <= 3) ? M2 : -1,
        value = rest > mine ? rest : mine
    };
};
// v * f where f = 2^k when e2 = k + 100000 (else e2 = 0): the exponent field
// moves on the integer pipes when v and the result are normal (the product is
// exact then, as the multiplication's would be); zeros, subnormals,
// infinities, NaNs and results outside the normal range take the FP64
// multiply.
XTG_DI double mul_pow2(double v, double f, int e2) {
    if (e2) {
        const long long b = __double_as_longlong(v);
        const int ef = (int)((b >> 52) & 0x7ff);
        const int e = ef + (e2 - 100000);
        if (ef != 0 && ef != 0x7ff && e >= 1 && e <= 2046)
            return __longlong_as_double(b + ((long long)(e2 - 100000) << 52));
    }
    return v * f;
}
template <int MODE, int K, class CT> XTG_DI void put_moment(CT& c, const RowParams& p, double sum, double sdev2) {
    if (MODE == 0) {
        RowFin<double>::put(c, K, sum);
    } else if (MODE == 1) {
        RowFin<double>::put(c, K, mul_pow2(sum, p.rdiv[K], p.rdiv_e2[K]));
    } else {
        const double var = mul_pow2(sdev2, p.vfac[K], p.vfac_e2[K]);  // (n * sum (x - mean)^2) / (n * divisor)
        RowFin<double>::put(c, K, MODE == 3 ? m_sqrt(var) : var);
    }
    if (K < 32) c.fixmask |= 1u << K;
}
template <class Sub, class... R> struct PutSameSub {
    template <class CT> static XTG_DI void run(CT&, const RowParams&, double, double) {}
};
template <class Sub, int K2, int M2, class C2, class S2, class... R> struct PutSameSub<Sub, RStat<K2, M2, C2, S2>, R...> {
    template <class CT> static XTG_DI void run(CT& c, const RowParams& p, double sum, double sdev2) {
        if constexpr (SameT<Sub, S2>::value && sizeof(C2) == 8 && M2 <= 3 && K2 < 32) put_moment<M2, K2>(c, p, sum, sdev2);
        PutSameSub<Sub, R...>::run(c, p, sum, sdev2);
    }
};

template <class LST> struct Stats;
template <> struct Stats<StatList<>> {
    template <int GROUP, int VEC, int NV, class RG, class CT>
    static XTG_DI void run(const RG (&)[NV], const bool (&)[NV][VEC], CT&, const RowParams&, void*) {}
};
template <int K, int MODE, class C, class Sub, class... Rest> struct Stats<StatList<RStat<K, MODE, C, Sub>, Rest...>> {
    template <int GROUP, int VEC, int NV, class RG, class CT>
    static XTG_DI void run(const RG (&rg)[NV], const bool (&ok)[NV][VEC], CT& c, const RowParams& p, void* smem) {
        typedef RowSum<GROUP, C> RS;
        typedef typename RS::A A;
        bool fixed_done = false;
        if constexpr (MODE <= 3 && sizeof(C) == 8) {
            if (K < 32 && ((c.fixmask >> K) & 1u)) {
                fixed_done = true;  // produced with an earlier statistic of the same operand
            } else {
                constexpr int later = SameSubMode<Sub, Rest...>::value;
                constexpr int MX = later > MODE ? later : MODE;
                double sum, sdev2;
                if (fixed_moments<GROUP, VEC, NV, MX, Sub>(rg, ok, c, p, smem, sum, sdev2)) {
                    fixed_done = true;
                    put_moment<MODE, K>(c, p, sum, sdev2);
                    PutSameSub<Sub, Rest...>::run(c, p, sum, sdev2);
                }
            }
        }
        if constexpr (MODE <= 3) {
            if (!fixed_done) {
                A s;
                RS::zero(s);
#pragma unroll
                for (int n = 0; n < NV; ++n)
#pragma unroll
                    for (int j = 0; j < VEC; ++j)
                        if (ok[n][j]) RS::add(s, cvt<C>(Sub::ev(rg[n], j, c)));
                s = group_reduce<GROUP>(s, reinterpret_cast<A*>(smem));
                s = bcast_group<GROUP>(s, reinterpret_cast<A*>(smem));
                // per-row scalar work in C's own precision (float rows never
                // touch the FP64 pipe; float64 rows multiply by host reciprocals)
                const C sum = RowFin<C>::total(s);
                if (MODE == 0) {
                    RowFin<C>::put(c, K, sum);
                } else if (MODE == 1) {
                    RowFin<C>::put(c, K, RowFin<C>::scale(sum, p, K));
                } else {
                    const C m = RowFin<C>::mean(sum, p);
                    A q;
                    RS::zero(q);
                    if constexpr (sizeof(C) == 4) {
                        // squared deviations are all >= 0 (no cancellation):
                        // four interleaved FP32 fma chains per lane (relative
                        // error below (n/(4*lanes) + 2) ulp), then compensated
                        // across lanes
                        float qa[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                        for (int n = 0; n < NV; ++n)
#pragma unroll
                            for (int j = 0; j < VEC; ++j)
                                if (ok[n][j]) {
                                    const float d = cvt<float>(Sub::ev(rg[n], j, c)) - m;
                                    qa[(n * VEC + j) & 3] = fmaf(d, d, qa[(n * VEC + j) & 3]);
                                }
                        q.hi = (qa[0] + qa[1]) + (qa[2] + qa[3]);
                    } else {
#pragma unroll
                        for (int n = 0; n < NV; ++n)
#pragma unroll
                            for (int j = 0; j < VEC; ++j)
                                if (ok[n][j]) RS::addsq(q, (C)(cvt<C>(Sub::ev(rg[n], j, c)) - m));
                    }
                    q = group_reduce<GROUP>(q, reinterpret_cast<A*>(smem));
                    q = bcast_group<GROUP>(q, reinterpret_cast<A*>(smem));
                    C var = RowFin<C>::scale(RowFin<C>::total(q), p, K);
                    if (var < C(0)) var = C(0);
                    RowFin<C>::put(c, K, MODE == 3 ? m_sqrt(var) : var);
                }
            }
        } else {
            AccSel<C, MODE == 4> a;
            a.start(MODE == 4 ? Lim<C>::lowest() : Lim<C>::maxv());
#pragma unroll
            for (int n = 0; n < NV; ++n)
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    if (ok[n][j]) a.add(cvt<C>(Sub::ev(rg[n], j, c)), (i64)((n * GROUP) + (int)(threadIdx.x % GROUP)) * VEC + j);
            a = group_reduce<GROUP>(a, reinterpret_cast<AccSel<C, MODE == 4>*>(smem));
            a = bcast_group<GROUP>(a, reinterpret_cast<AccSel<C, MODE == 4>*>(smem));
            c.stat[K] = (double)a.value();
            c.statf[K] = (float)a.value();
        }
        Stats<StatList<Rest...>>::template run<GROUP, VEC, NV>(rg, ok, c, p, smem);
    }
};

// FULL: row_len == NV * group size * VEC, so no element needs a bounds mask.
template <class Tree, class SL, class LS, class OutT, int VEC, int NV, int GROUP, int RO, int NSTAT, int FULL>
__global__ void __launch_bounds__(256) k_rowfused(const RowParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    __shared__ __align__(16) unsigned char smem_raw[32 * 48];
    Ctx<NSTAT> c;
    c.scal = p.scal;
    const int gsz = GROUP <= 32 ? 32 : (int)blockDim.x;
    const int gpb = (int)blockDim.x / gsz;
    const int gt = (int)threadIdx.x % gsz;
    const i64 gid = (i64)blockIdx.x * gpb + (int)threadIdx.x / gsz;
    const i64 ng = (i64)gridDim.x * gpb;
    for (i64 row = gid; row < p.n_rows; row += ng) {
        i64 ko[RO];
        decode_dims<RO, true>(p.oshape, (const FastDiv*)0, row, ko);
        i64 base[XTG_KMAX_LEAVES];
#pragma unroll
        for (int l = 0; l < LS::N; ++l) {
            i64 o = 0;
#pragma unroll
            for (int d = 0; d < RO; ++d) o += ko[d] * p.lo[l][d];
            base[l] = o;
        }
        RG rg[NV];
        bool ok[NV][VEC];
#pragma unroll
        for (int n = 0; n < NV; ++n) {
            const i64 e0 = ((i64)n * gsz + gt) * VEC;
#pragma unroll
            for (int j = 0; j < VEC; ++j) ok[n][j] = FULL || (e0 + j) < p.row_len;
            if (FULL || e0 < p.row_len) {
                i64 off[XTG_KMAX_LEAVES];
#pragma unroll
                for (int l = 0; l < LS::N; ++l) off[l] = base[l] + e0 * p.li[l];
                LoadLeavesAt<LS>::template run<VEC>(rg[n], p.leaf, off, p.li);
            }
        }
        c.fixmask = 0;
        Stats<SL>::template run<GROUP, VEC, NV>(rg, ok, c, p, (void*)smem_raw);
        Prep<Tree>::run(rg[0], c);
        i64 ob = 0;
#pragma unroll
        for (int d = 0; d < RO; ++d) ob += ko[d] * p.oo[d];
#pragma unroll
        for (int n = 0; n < NV; ++n) {
            const i64 e0 = ((i64)n * gsz + gt) * VEC;
            if (FULL || e0 < p.row_len) {
                OutT v[VEC];
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[j] = cvt<OutT>(Tree::ev(rg[n], j, c));
                st_out<OutT, K_CONTIG, VEC>(reinterpret_cast<OutT*>(p.out), ob + e0 * p.oi, p.oi, v);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// K7 with bulk copies.  Each warp owns rows; the rows of every leaf stream
// into a per-warp buffer in shared memory (one, or a double buffer) with one
// cp.async.bulk per leaf per row (the TMA engine's 1-D bulk copy, completion
// counted in bytes on an mbarrier), issued one row ahead, so HBM reads of row
// i+1 overlap the statistics and the stores of row i.  Requires every leaf to
// be contiguous along the row, rows 16-byte aligned and a multiple of 16
// bytes.
XTG_DI unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
XTG_DI void mbar_init(u64* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
XTG_DI void mbar_expect_tx(u64* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
XTG_DI bool mbar_try_wait(u64* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
XTG_DI void bulk_g2s(void* dst, const void* src, unsigned bytes, u64* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
XTG_DI void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
XTG_DI void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
XTG_DI void mbar_arrive(u64* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Named barrier 1 over the first NT threads of the block (the consumer warps
// of a kernel whose last warp is a producer that never joins it).
template <int NT> XTG_DI void bar_sync_n() { asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory"); }
template <int NT> XTG_DI bool bar_or_n(bool v) {
    unsigned r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((unsigned)v), "n"(NT)
        : "memory");
    return r != 0;
}

// K13: a full reduction of one contiguous leaf streamed through shared
// memory.  Each block walks its work items (the same fixed partition as K3),
// each item in stages of 1024 16-byte vectors.  The block's last warp is the
// producer: its lane 0 copies every stage with cp.async.bulk into a ring of
// NS buffers, completion on the slot's "full" mbarrier, and reuses a slot
// once the 8 consumer warps have arrived on its "empty" mbarrier — consumer
// warps never wait for one another between stages.  Consumer thread t folds
// vectors t, t + 256, t + 512, t + 768 of every stage of its item (the
// vectors and the order of K3 with a 256-thread group) and the consumers
// combine with K3's tree, so results equal K3's bit for bit.
// Every wait is bounded.  A consumer warp that gives up stops arriving (so
// the slot is never refilled under it); at the end of the item the
// consumers decide together, set the error word and return.  The producer
// gives up when a slot is not released in time, and before it returns it
// waits (bounded) for its copies still in flight, so the block's shared
// memory outlives every copy.
template <class T> struct SmemVec16 {
    template <int VEC> static XTG_DI void get(T (&dst)[VEC], const unsigned char* p) {
        union {
            uint4 q;
            T e[VEC];
        } u;
        u.q = *reinterpret_cast<const uint4*>(p);
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = u.e[j];
    }
};
// K3's block tree (group_reduce<256>) over the 256 consumer threads.
template <class A> XTG_DI A consumer_reduce(A a, A* smem) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        A o = shfl_xor_pod(a, m);
        a.merge(o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bar_sync_n<256>();
    if (lane == 0) smem[warp] = a;
    bar_sync_n<256>();
    if (threadIdx.x == 0) {
        A r = smem[0];
        for (int w = 1; w < 8; ++w) r.merge(smem[w]);
        a = r;
    }
    return a;
}
template <class Tree, class LS, class TL, class Acc, class Out, int POST, int VEC, int NS>
__global__ void __launch_bounds__(288) k_reduce_stream(const RedParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    constexpr unsigned SB = 16384;  // stage bytes: 1024 vectors
    constexpr int kPolls = 1 << 22;
    extern __shared__ __align__(128) unsigned char sbuf[];
    __shared__ u64 full[NS], empty[NS];
    __shared__ Acc smem[8];
    const int tid = (int)threadIdx.x;
    const i64 nitems = p.nsplit;
    const char* base = reinterpret_cast<const char*>(p.leaf[0]);
    auto item_len = [&](i64 w) -> i64 {
        const i64 rb = w * p.chunk;
        const i64 re = rb + p.chunk < p.n_redv ? rb + p.chunk : p.n_redv;
        return re - rb;
    };
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 8);
        }
        fence_mbar_init();
    }
    __syncthreads();
    if (tid >= 256) {
        // the producer (lane 0 of the last warp)
        if (tid != 256) return;
        i64 q = 0;
        bool stop = false;
        for (i64 w = blockIdx.x; w < nitems && !stop; w += gridDim.x) {
            const i64 len = item_len(w);
            for (i64 v0 = 0; v0 < len; v0 += 1024) {
                const int slot = (int)(q % NS);
                if (q >= NS) {
                    const unsigned par = (unsigned)(((q / NS) - 1) & 1);
                    bool ok = false;
                    for (int k = 0; k < kPolls; ++k)
                        if (mbar_try_wait(&empty[slot], par)) {
                            ok = true;
                            break;
                        }
                    if (!ok) {
                        stop = true;
                        break;
                    }
                }
                const i64 nv = len - v0 < 1024 ? len - v0 : 1024;
                const unsigned bytes = (unsigned)(nv * 16);
                if (q >= NS) fence_proxy_async_smem();  // the consumers' reads before the copy's writes
                mbar_expect_tx(&full[slot], bytes);
                bulk_g2s(sbuf + (size_t)slot * SB, base + (w * p.chunk + v0) * 16, bytes, &full[slot]);
                ++q;
            }
        }
        // the copies that may still be in flight: the last issued stage of each slot
        bool drained = true;
        for (i64 r = q > NS ? q - NS : 0; r < q; ++r) {
            bool ok = false;
            for (int k = 0; k < kPolls; ++k)
                if (mbar_try_wait(&full[r % NS], (unsigned)((r / NS) & 1))) {
                    ok = true;
                    break;
                }
            drained = drained && ok;
        }
        if (stop || !drained) atomicExch(p.err, 1);
        return;
    }
    // the 256 consumers
    Ctx<0> c;
    c.scal = p.scal;
    i64 q = 0;
    bool bad = false;
    for (i64 w = blockIdx.x; w < nitems; w += gridDim.x) {
        Acc acc;
        acc.init(p);
        if (NeedsShift<Acc>::value && p.n_red > 0) {
            typename LS::template R<1>::type rg1;
            i64 off[XTG_KMAX_LEAVES] = {0};
            i64 inner[XTG_KMAX_LEAVES] = {1};
            LoadLeavesAt<LS>::template run<1>(rg1, p.leaf, off, inner);
            Shift<Acc>::set(acc, Tree::ev(rg1, 0, c));
        }
        typename Work<Acc>::T wa;
        wa.from(acc);
        const i64 len = item_len(w);
        const i64 ns = (len + 1023) / 1024;
        for (i64 s = 0; s < ns; ++s, ++q) {
            const int slot = (int)(q % NS);
            if (!bad) {
                const unsigned par = (unsigned)((q / NS) & 1);
                bool ok = false;
                for (int k = 0; k < kPolls; ++k)
                    if (mbar_try_wait(&full[slot], par)) {
                        ok = true;
                        break;
                    }
                bad = !ok;
            }
            if (!bad) {
                const unsigned char* buf = sbuf + (size_t)slot * SB;
                const i64 nvs = len - s * 1024 < 1024 ? len - s * 1024 : 1024;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int v = tid + 256 * j;
                    if (v < nvs) {
                        RG rg;
                        SmemVec16<TL>::template get<VEC>(RegAt<0>::get(rg), buf + (size_t)v * 16);
                        AddVec<HasAdd2<typename Work<Acc>::T>::value != 0>::template run<VEC, Tree>(
                            wa, rg, (w * p.chunk + s * 1024 + v) * VEC, c);
                    }
                }
            }
            // every lane has read the slot: the warp releases it
            if (__any_sync(0xffffffffu, bad)) bad = true;
            __syncwarp();
            if (!bad && (tid & 31) == 0) mbar_arrive(&empty[slot]);
        }
        wa.to(acc);
        if (bar_or_n<256>(bad)) {
            if (tid == 0) atomicExch(p.err, 1);
            return;
        }
        acc = consumer_reduce(acc, smem);
        if (tid == 0) {
            if (p.nsplit > 1) reinterpret_cast<Acc*>(p.partial)[w] = acc;
            else Store<Out, Acc, POST>::put(acc, p, 0);
        }
        bar_sync_n<256>();  // smem is reused by the next item's combine
    }
}


template <class T, int VEC>
XTG_DI void ld_smem(T (&dst)[VEC], const T* p) {
    const int B = (int)sizeof(T) * VEC;
    if (B == 16 || B == 8 || B == 4) {
        typedef typename VecT<B>::t V;
        union { V v; T e[VEC]; } u;
        u.v = *reinterpret_cast<const V*>(p);
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = u.e[j];
    } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) dst[j] = p[j];
    }
}
template <int I, int VEC, class... S> struct SmemLoad;
template <int I, int VEC> struct SmemLoad<I, VEC> {
    template <class RG> static XTG_DI void run(RG&, const unsigned char*, const unsigned*, i64) {}
};
template <int I, int VEC, class S0, class... S> struct SmemLoad<I, VEC, S0, S...> {
    template <class RG> static XTG_DI void run(RG& rg, const unsigned char* buf, const unsigned* loff, i64 e0) {
        typedef typename S0::type T;
        ld_smem<T, VEC>(rg.v, reinterpret_cast<const T*>(buf + loff[I]) + e0);
        SmemLoad<I + 1, VEC, S...>::run(rg.rest, buf, loff, e0);
    }
};
template <class LS> struct LoadRowSmem;
template <class... S> struct LoadRowSmem<LeafSet<S...>> {
    template <int VEC, class RG> static XTG_DI void run(RG& rg, const unsigned char* buf, const unsigned* loff, i64 e0) {
        SmemLoad<0, VEC, S...>::run(rg, buf, loff, e0);
    }
};

// NB = 2: a double buffer per warp, row i + 1 copied while row i is reduced
// from shared memory.  NB = 1: one buffer per warp, refilled with row i + 1
// as soon as row i sits in registers (half the shared memory, so more warps
// per SM).  MINB: the launch-bounds minimum of resident blocks per SM.
template <class Tree, class SL, class LS, class OutT, int VEC, int NV, int RO, int NSTAT, int FULL, int NB = 2, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) k_rowfused_tma(const RowParams p) {
    pdl_wait();
    typedef typename LS::template R<VEC>::type RG;
    extern __shared__ __align__(128) unsigned char dsmem[];
    __shared__ __align__(16) unsigned char red_smem[32 * 48];
    __shared__ u64 bars[8];
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int nw = (int)blockDim.x >> 5;
    u64* mybar = bars + 2 * warp;
    unsigned char* const buf0 = dsmem + (size_t)(NB * warp) * p.buf_bytes;  // buffer b at buf0 + b * buf_bytes
    if (lane == 0) {
        mbar_init(&mybar[0], 1);
        mbar_init(&mybar[1], 1);
        fence_mbar_init();
    }
    __syncwarp();
    Ctx<NSTAT> c;
    c.scal = p.scal;
    const i64 gid = (i64)blockIdx.x * nw + warp;
    const i64 ng = (i64)gridDim.x * nw;
    auto issue = [&](i64 row, int b) {
        if (lane == 0) {
            i64 ko[RO];
            decode_dims<RO, true>(p.oshape, (const FastDiv*)0, row, ko);
            mbar_expect_tx(&mybar[b], p.buf_bytes);
#pragma unroll
            for (int l = 0; l < LS::N; ++l) {
                i64 o = 0;
#pragma unroll
                for (int d = 0; d < RO; ++d) o += ko[d] * p.lo[l][d];
                const unsigned char* src = reinterpret_cast<const unsigned char*>(p.leaf[l]) + o * (p.lbytes[l] / p.row_len);
                bulk_g2s(buf0 + (size_t)b * p.buf_bytes + p.loff[l], src, p.lbytes[l], &mybar[b]);
            }
        }
    };
    int it = 0;
    if (gid < p.n_rows) issue(gid, 0);
    for (i64 row = gid; row < p.n_rows; row += ng, ++it) {
        const int b = NB == 2 ? (it & 1) : 0;
        if (NB == 2 && row + ng < p.n_rows) issue(row + ng, b ^ 1);
        const unsigned parity = NB == 2 ? ((unsigned)(it >> 1) & 1u) : ((unsigned)it & 1u);
        bool done = false;
        for (int k = 0; k < (1 << 22); ++k) {
            if (mbar_try_wait(&mybar[b], parity)) {
                done = true;
                break;
            }
        }
        // one decision for the whole warp: a lane that gave up must not
        // leave while the others go on into full-mask shuffles
        done = __all_sync(0xffffffffu, done);
        if (!done) {
            // give up: flag it, wait (bounded) for the copy into the other
            // buffer if one was issued, and leave.  The copy that timed out
            // may still be in flight into this block's shared memory when
            // the block exits; the error word tells the host that the
            // launch's results (and the device state) are not to be trusted.
            if (lane == 0) atomicExch(p.err, 1);
            if (NB == 2 && row + ng < p.n_rows) {
                const unsigned par2 = (unsigned)((it + 1) >> 1) & 1u;
                for (int k = 0; k < (1 << 22); ++k)
                    if (mbar_try_wait(&mybar[b ^ 1], par2)) break;
            }
            return;
        }
        RG rg[NV];
        bool ok[NV][VEC];
#pragma unroll
        for (int n = 0; n < NV; ++n) {
            const i64 e0 = ((i64)n * 32 + lane) * VEC;
#pragma unroll
            for (int j = 0; j < VEC; ++j) ok[n][j] = FULL || (e0 + j) < p.row_len;
            if (FULL || e0 < p.row_len) LoadRowSmem<LS>::template run<VEC>(rg[n], buf0 + (size_t)b * p.buf_bytes, p.loff, e0);
        }
        if (NB == 1) {
            // the row is in registers: refill the buffer with the next one
            fence_proxy_async_smem();
            __syncwarp();
            if (row + ng < p.n_rows) issue(row + ng, 0);
        }
        c.fixmask = 0;
        Stats<SL>::template run<32, VEC, NV>(rg, ok, c, p, (void*)red_smem);
        Prep<Tree>::run(rg[0], c);
        i64 ko[RO];
        decode_dims<RO, true>(p.oshape, (const FastDiv*)0, row, ko);
        i64 ob = 0;
#pragma unroll
        for (int d = 0; d < RO; ++d) ob += ko[d] * p.oo[d];
#pragma unroll
        for (int n = 0; n < NV; ++n) {
            const i64 e0 = ((i64)n * 32 + lane) * VEC;
            if (FULL || e0 < p.row_len) {
                OutT v[VEC];
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[j] = cvt<OutT>(Tree::ev(rg[n], j, c));
                st_out<OutT, K_CONTIG, VEC>(reinterpret_cast<OutT*>(p.out), ob + e0, 1, v);
            }
        }
        if (NB == 2) {
            // all lanes are done reading buffer b before it is refilled
            fence_proxy_async_smem();
            __syncwarp();
        }
    }
}

// a * (1 / b) with b invariant over a row: the reciprocal is computed once
// per row (Prep) into statistic slot KR (a division costs ~10 FP64
// operations on GB300, and an IEEE FP32 division several instructions).
template <class T, class A, class B, int KR> struct MulRecip {
    typedef T type;
    template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C& c) {
        return cvt<T>(A::ev(r, j, c)) * StatGet<T>::get(c, KR);
    }
};
template <class T, class A, class B, int KR> struct Prep<MulRecip<T, A, B, KR>> {
    template <class RG, class C> static XTG_DI void run(const RG& r, C& c) {
        Prep<A>::run(r, c);
        Prep<B>::run(r, c);
        StatGet<T>::put(c, KR, T(1) / cvt<T>(B::ev(r, 0, c)));
    }
};

// ---------------------------------------------------------------------------
// K8: batched persistent kernels.  Thousands of instances of one tree with
// uneven (rows, cols) run in ONE launch: CTAs pull tiles (a run of rows of
// one instance, sized to about the same number of elements) from a device
// counter until the list is exhausted; a sub-warp group of GL lanes owns a
// row.  Row reductions: each row's result is produced by one group in a fixed
// order, so results do not depend on which CTA took the tile.
// Row loads for the vector form of K8: per leaf a 2-bit mode for the row —
// 3: contiguous and 16-byte aligned at the row's vector start (one vector
// load), 1: contiguous but differently aligned (VEC scalar loads), 0:
// broadcast along the row (one load).  The modes are uniform over a row, so
// the branches do not diverge.
template <int I, int VEC, class... S> struct LoadRowV;
template <int I, int VEC> struct LoadRowV<I, VEC> {
    template <class RG> static XTG_DI void run(RG&, const void* const*, i64, unsigned) {}
};
template <int I, int VEC, class S0, class... S> struct LoadRowV<I, VEC, S0, S...> {
    template <class RG> static XTG_DI void run(RG& rg, const void* const* ptr, i64 col, unsigned modes) {
        typedef typename S0::type T;
        const T* b = reinterpret_cast<const T*>(ptr[I]);
        const unsigned m = (modes >> (2 * I)) & 3u;
        if (VEC > 1 && m == 3u) {
            ld_contig<T, VEC>(rg.v, b + col);
        } else if (m != 0u) {
#pragma unroll
            for (int j = 0; j < VEC; ++j) rg.v[j] = ld1<T>(b + col + j);
        } else {
            const T v = ld1<T>(b);
#pragma unroll
            for (int j = 0; j < VEC; ++j) rg.v[j] = v;
        }
        LoadRowV<I + 1, VEC, S...>::run(rg.rest, ptr, col, modes);
    }
};
template <class LS> struct LoadRowVec;
template <class... S> struct LoadRowVec<LeafSet<S...>> {
    template <int VEC, class RG> static XTG_DI void run(RG& rg, const void* const* ptr, i64 col, unsigned modes) {
        LoadRowV<0, VEC, S...>::run(rg, ptr, col, modes);
    }
};

// K8 vector form: every leaf of every instance is contiguous (column stride
// 1) or broadcast (0) along a row, all of one element size E = 16 / VEC.  A
// group of GL lanes owns a row: a scalar head up to the first 16-byte
// boundary of the row's first contiguous leaf, then VEC-wide vectors (16-byte
// loads for the leaves aligned like it, scalar loads for the others), then a
// scalar tail; U vectors per lane in flight.  Each lane folds its columns in
// order; lanes merge by the fixed butterfly, so a row's result does not
// depend on the tile's CTA.
template <class Tree, class LS, class Acc, class Out, int POST, int GL, int U, int VEC>
XTG_DI void batch_row_vec(const BatchInst* I, i64 row, int gl, Acc& acc, Ctx<0>& c) {
    typedef typename LS::template R<VEC>::type RGV;
    typedef typename LS::template R<1>::type RG1;
    const i64 cols = I->cols;
    const void* rp[XTG_KMAX_LEAVES];
    unsigned modes = 0;
    unsigned long long prim = ~0ull;  // address of the first contiguous leaf's row
#pragma unroll
    for (int l = 0; l < LS::N; ++l) {
        rp[l] = reinterpret_cast<const char*>(I->leaf[l]) + row * I->rs[l] * (16 / VEC);
        if (I->cs[l] != 0) {
            modes |= 1u << (2 * l);
            if (prim == ~0ull) prim = (unsigned long long)rp[l];
        }
    }
    i64 head = 0;
    if (prim != ~0ull) {
        const unsigned mis = (unsigned)(prim & 15u) / (16 / VEC);
        head = mis ? (i64)(VEC - mis) : 0;
        if (head > cols) head = cols;
#pragma unroll
        for (int l = 0; l < LS::N; ++l)
            if (I->cs[l] != 0 && (((unsigned long long)rp[l] + (unsigned long long)head * (16 / VEC)) & 15u) == 0) modes |= 2u << (2 * l);
    }
    if (NeedsShift<Acc>::value && cols > 0) {
        RG1 r1;
        LoadRowVec<LS>::template run<1>(r1, rp, 0, modes & 0x55555555u);
        Shift<Acc>::set(acc, Tree::ev(r1, 0, c));
    }
    // head (fewer than VEC columns)
    if (gl < head) {
        RG1 r1;
        LoadRowVec<LS>::template run<1>(r1, rp, gl, modes & 0x55555555u);
        acc.add(Tree::ev(r1, 0, c), (i64)gl);
    }
    const i64 nv = (cols - head) / VEC;
    for (i64 v0 = gl; v0 < nv; v0 += (i64)GL * U) {
        RGV rg[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const i64 v = v0 + (i64)u * GL;
            if (v < nv) LoadRowVec<LS>::template run<VEC>(rg[u], rp, head + v * VEC, modes);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const i64 v = v0 + (i64)u * GL;
            if (v < nv) {
#pragma unroll
                for (int j = 0; j < VEC; ++j) acc.add(Tree::ev(rg[u], j, c), head + v * VEC + j);
            }
        }
    }
    // tail
    const i64 t0 = head + nv * VEC;
    if (t0 + gl < cols) {
        RG1 r1;
        LoadRowVec<LS>::template run<1>(r1, rp, t0 + gl, modes & 0x55555555u);
        acc.add(Tree::ev(r1, 0, c), t0 + gl);
    }
}

template <class Tree, class LS, class Acc, class Out, int POST, int GL, int U, int VEC = 1, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) k_batch_rowreduce(const BatchParams p) {
    pdl_wait();
    typedef typename LS::template R<1>::type RG;
    __shared__ i64 s_tile;
    Ctx<0> c;
    c.scal = p.scal;
    // the vector form takes tiles per warp (no block barrier between tiles);
    // the strided form per block
    constexpr bool WT = VEC > 1;
    const int lane32 = (int)threadIdx.x & 31;
    const int g = WT ? lane32 / GL : (int)threadIdx.x / GL, gl = (int)threadIdx.x % GL;
    const int ngroups = WT ? 32 / GL : (int)blockDim.x / GL;
    FinP fp;
    fp.init_f = p.init_f;
    fp.init_i = p.init_i;
    fp.has_initial = p.has_initial;
    fp.initial_f = p.initial_f;
    fp.initial_i = p.initial_i;
    for (;;) {
        i64 t;
        if (WT) {
            int tt = 0;
            if (lane32 == 0) tt = atomicAdd(p.counter, 1);
            t = (i64)__shfl_sync(0xffffffffu, tt, 0);
        } else {
            __syncthreads();
            if (threadIdx.x == 0) s_tile = (i64)atomicAdd(p.counter, 1);
            __syncthreads();
            t = s_tile;
        }
        if (t >= p.ntiles) break;
        const BatchTile tl = p.tiles[t];
        const BatchInst* I = p.inst + tl.inst;
        const i64 cols = I->cols;
        fp.divisor = I->divisor;
        fp.n_red = cols;
        i64 cs[XTG_KMAX_LEAVES], rsv[XTG_KMAX_LEAVES];
#pragma unroll
        for (int l = 0; l < LS::N; ++l) {
            cs[l] = I->cs[l];
            rsv[l] = I->rs[l];
        }
        for (int r0 = 0; r0 < tl.nrows; r0 += ngroups) {
            const int r = r0 + g;
            const bool active = r < tl.nrows;
            const i64 row = tl.row0 + r;
            Acc acc;
            acc.init(fp);
            if (VEC > 1) {
                if (active) batch_row_vec<Tree, LS, Acc, Out, POST, GL, U, VEC>(I, row, gl, acc, c);
            } else if (active) {
                i64 base[XTG_KMAX_LEAVES];
#pragma unroll
                for (int l = 0; l < LS::N; ++l) base[l] = row * rsv[l];
                if (NeedsShift<Acc>::value && cols > 0) {
                    RG r1;
                    LoadLeavesAt<LS>::template run<1>(r1, I->leaf, base, cs);
                    Shift<Acc>::set(acc, Tree::ev(r1, 0, c));
                }
                for (i64 c0 = gl; c0 < cols; c0 += (i64)GL * U) {
                    RG rg[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const i64 col = c0 + (i64)u * GL;
                        if (col < cols) {
                            i64 off[XTG_KMAX_LEAVES];
#pragma unroll
                            for (int l = 0; l < LS::N; ++l) off[l] = base[l] + col * cs[l];
                            LoadLeavesAt<LS>::template run<1>(rg[u], I->leaf, off, cs);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const i64 col = c0 + (i64)u * GL;
                        if (col < cols) acc.add(Tree::ev(rg[u], 0, c), col);
                    }
                }
            }
#pragma unroll
            for (int m = GL / 2; m >= 1; m >>= 1) {
                Acc o = shfl_xor_pod(acc, m);
                acc.merge(o);
            }
            if (active && gl == 0) reinterpret_cast<Out*>(I->out)[row * I->ors] = finish<Out, Acc, POST>(acc, fp);
        }
    }
}

template <class Tree, class LS, class OutT, int GL, int U>
__global__ void __launch_bounds__(256) k_batch_assign(const BatchParams p) {
    pdl_wait();
    typedef typename LS::template R<1>::type RG;
    __shared__ i64 s_tile;
    Ctx<0> c;
    c.scal = p.scal;
    const int g = (int)threadIdx.x / GL, gl = (int)threadIdx.x % GL, ngroups = (int)blockDim.x / GL;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = (i64)atomicAdd(p.counter, 1);
        __syncthreads();
        const i64 t = s_tile;
        if (t >= p.ntiles) break;
        const BatchTile tl = p.tiles[t];
        const BatchInst* I = p.inst + tl.inst;
        const i64 cols = I->cols;
        for (int r = g; r < tl.nrows; r += ngroups) {
            const i64 row = tl.row0 + r;
            i64 base[XTG_KMAX_LEAVES], cs[XTG_KMAX_LEAVES];
#pragma unroll
            for (int l = 0; l < LS::N; ++l) {
                base[l] = row * I->rs[l];
                cs[l] = I->cs[l];
            }
            OutT* out = reinterpret_cast<OutT*>(I->out) + row * I->ors;
            for (i64 c0 = gl; c0 < cols; c0 += (i64)GL * U) {
                RG rg[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const i64 col = c0 + (i64)u * GL;
                    if (col < cols) {
                        i64 off[XTG_KMAX_LEAVES];
#pragma unroll
                        for (int l = 0; l < LS::N; ++l) off[l] = base[l] + col * cs[l];
                        LoadLeavesAt<LS>::template run<1>(rg[u], I->leaf, off, cs);
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const i64 col = c0 + (i64)u * GL;
                    if (col < cols) out[col * I->ocs] = cvt<OutT>(Tree::ev(rg[u], 0, c));
                }
            }
        }
    }
}

// (a - m) / b with m and b invariant over a row, as one fused multiply-add
// per element: a * r - m * r with r = 1 / b; r (slot KR) and m * r (slot KM)
// are computed once per row (Prep).
template <class T, class A, class M, class B, int KR, int KM> struct FmaRecipSub {
    typedef T type;
    template <class RG, class C> static XTG_DI T ev(const RG& r, int j, const C& c) {
        return fma(cvt<T>(A::ev(r, j, c)), StatGet<T>::get(c, KR), -StatGet<T>::get(c, KM));
    }
};
template <class T, class A, class M, class B, int KR, int KM> struct Prep<FmaRecipSub<T, A, M, B, KR, KM>> {
    template <class RG, class C> static XTG_DI void run(const RG& r, C& c) {
        Prep<A>::run(r, c);
        Prep<M>::run(r, c);
        Prep<B>::run(r, c);
        const T rb = T(1) / cvt<T>(B::ev(r, 0, c));
        StatGet<T>::put(c, KR, rb);
        StatGet<T>::put(c, KM, cvt<T>(M::ev(r, 0, c)) * rb);
    }
};
// float64 (a - m) / sqrt(v): 1 / sqrt(v) by CUDA's rsqrt (within 1 ulp) instead
// of a correctly rounded sqrt and division — each lane of a warp runs this
// once per row, at GB300's FP64 rate.
template <class A, class M, class X, int KR, int KM> struct Prep<FmaRecipSub<double, A, M, Sqrt<double, X>, KR, KM>> {
    template <class RG, class C> static XTG_DI void run(const RG& r, C& c) {
        Prep<A>::run(r, c);
        Prep<M>::run(r, c);
        Prep<X>::run(r, c);
        const double rb = rsqrt(cvt<double>(X::ev(r, 0, c)));
        StatGet<double>::put(c, KR, rb);
        StatGet<double>::put(c, KM, cvt<double>(M::ev(r, 0, c)) * rb);
    }
};

}  // namespace xtg
#endif
