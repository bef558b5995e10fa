// xt.hpp — header-only C++ surface of the GB300 evaluator.
//
// Existing xtensor call sites compile against it unchanged: xt::xarray<T>,
// xt::xtensor<T, N>, arithmetic / math operators building lazy expression
// trees (xfunction), xt::sum / prod / amax / amin / mean / variance /
// stddev / norm_* with axes, keep_dims, initial and evaluation_strategy,
// xt::argmax / argmin, xt::cumsum / cumprod / nancumsum / nancumprod,
// xt::index_view / filter / filtration / masked_view (read and write),
// xt::transpose / strided views / xt::view slices,
// xt::noalias, xt::eval.  Containers live in device memory; assigning an
// expression lowers its template tree to the C ABI (include/xtg.h) and one
// fused sm_103a kernel evaluates it.  Reading an element copies it back
// (after the stream has finished the work that produced it).
//
// Semantics restated from xtensor 0.27.1: expression result types follow the
// functors' decltype (include/xtensor/core/xoperation.hpp:30-143,
// core/xmath.hpp:84-99, 295-341); reducer result types and options follow
// XTENSOR_REDUCER_FUNCTION (core/xmath.hpp:367-423) and reducer_options
// (reducers/xreducer.hpp:35-161); `a = e` evaluates into a temporary when e
// refers to a (xsemantic.hpp:620-640), `noalias(a) = e` assigns in place
// (core/xnoalias.hpp:19-230); errors are the reference's exceptions
// (broadcast_error, std::runtime_error for axes, std::out_of_range).
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <istream>
#include <iterator>
#include <memory>
#include <numeric>
#include <ostream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../xtg.h"

namespace xt {

// ---------------------------------------------------------------------------- errors
class broadcast_error : public std::runtime_error {
public:
    explicit broadcast_error(const char* m) : std::runtime_error(m) {}
};

namespace detail {
inline void check(xtg_status s) {
    if (s == XTG_OK) return;
    const char* m = xtg_last_error();
    switch (s) {
        case XTG_ERR_BROADCAST: throw broadcast_error(m);
        case XTG_ERR_OUT_OF_RANGE: throw std::out_of_range(m);
        case XTG_ERR_AXIS: throw std::runtime_error(m);
        default: throw std::runtime_error(std::string(xtg_status_string(s)) + ": " + m);
    }
}

template <class T> struct dtype_of;
template <> struct dtype_of<bool> { static constexpr int value = XTG_BOOL; };
template <> struct dtype_of<int8_t> { static constexpr int value = XTG_INT8; };
template <> struct dtype_of<uint8_t> { static constexpr int value = XTG_UINT8; };
template <> struct dtype_of<int16_t> { static constexpr int value = XTG_INT16; };
template <> struct dtype_of<uint16_t> { static constexpr int value = XTG_UINT16; };
template <> struct dtype_of<int32_t> { static constexpr int value = XTG_INT32; };
template <> struct dtype_of<uint32_t> { static constexpr int value = XTG_UINT32; };
template <> struct dtype_of<long> { static constexpr int value = XTG_INT64; };
template <> struct dtype_of<unsigned long> { static constexpr int value = XTG_UINT64; };
template <> struct dtype_of<long long> { static constexpr int value = XTG_INT64; };
template <> struct dtype_of<unsigned long long> { static constexpr int value = XTG_UINT64; };
template <> struct dtype_of<float> { static constexpr int value = XTG_FLOAT32; };
template <> struct dtype_of<double> { static constexpr int value = XTG_FLOAT64; };

inline xtg_stream& current_stream() {
    static thread_local xtg_stream s = nullptr;
    return s;
}

// Postfix lowering of a template tree.
struct lowering {
    xtg_expr e;
    std::vector<const void*> ids;
    std::vector<std::shared_ptr<void>> temps;  // evaluated sub-reductions
    std::vector<const xtg_chunked*> chunked;   // per leaf: its chunked array, or null
    lowering() { std::memset(&e, 0, sizeof e); }
    int leaf(const xtg_array& a, const void* id) {
        for (size_t i = 0; i < ids.size(); ++i)
            if (ids[i] == id && e.leaves[i].data == a.data && e.leaves[i].rank == a.rank) return (int)i;
        if (e.n_leaves >= XTG_MAX_LEAVES) throw std::runtime_error("xt: more than 8 distinct leaves in one expression");
        e.leaves[e.n_leaves] = a;
        ids.push_back(id);
        chunked.push_back(nullptr);
        return e.n_leaves++;
    }
    // a chunked array as a leaf: `a` is its stand-in (dtype, shape)
    int chunked_leaf(const xtg_array& a, const void* id, const xtg_chunked* c) {
        const int i = leaf(a, id);
        chunked[(size_t)i] = c;
        return i;
    }
    bool has_chunked() const {
        for (const xtg_chunked* c : chunked)
            if (c) return true;
        return false;
    }
    // the tree is one chunked leaf
    const xtg_chunked* only_chunked() const { return e.n_nodes == 1 && e.n_leaves == 1 ? chunked[0] : nullptr; }
    void node(int op, int dtype, int arg = 0, int aux = 0, xtg_value imm = xtg_value{0.0}) {
        if (e.n_nodes >= XTG_MAX_NODES) throw std::runtime_error("xt: expression tree too large");
        xtg_node& n = e.nodes[e.n_nodes++];
        n.op = op;
        n.dtype = dtype;
        n.arg = arg;
        n.aux = aux;
        n.imm = imm;
    }
};
// Consumers that take dense leaves only: each chunked leaf is read into a
// dense device temporary (xtg_chunked_to_dense) that lives with the lowering.
inline void resolve_chunked(lowering& L) {
    for (int i = 0; i < L.e.n_leaves; ++i) {
        const xtg_chunked* c = L.chunked[(size_t)i];
        if (!c) continue;
        static const int sz[XTG_NUM_DTYPES] = {1, 1, 1, 2, 2, 4, 4, 8, 8, 2, 4, 8};
        int64_t n = 1;
        for (int d = 0; d < c->rank; ++d) n *= c->shape[d];
        void* p = nullptr;
        check(xtg_malloc(&p, (size_t)std::max<int64_t>(n * sz[c->dtype], 16), current_stream()));
        std::shared_ptr<void> hold(p, [](void* q) { xtg_free(q, current_stream()); });
        xtg_array d = L.e.leaves[i];
        d.data = p;
        check(xtg_chunked_to_dense(c, &d, current_stream()));
        L.e.leaves[i] = d;
        L.chunked[(size_t)i] = nullptr;
        L.temps.push_back(hold);
    }
}
}  // namespace detail

inline void set_stream(xtg_stream s) { detail::current_stream() = s; }

// ---------------------------------------------------------------------------- expressions
template <class D> class xexpression {
public:
    const D& derived_cast() const& noexcept { return *static_cast<const D*>(this); }
    D& derived_cast() & noexcept { return *static_cast<D*>(this); }
};

template <class E> struct is_xexpression : std::is_base_of<xexpression<std::decay_t<E>>, std::decay_t<E>> {};

using dynamic_shape_t = std::vector<std::size_t>;
template <class T> using dynamic_shape = std::vector<T>;

// a scalar operand (xscalar)
template <class T> class xscalar : public xexpression<xscalar<T>> {
public:
    using value_type = T;
    explicit xscalar(T v) : m_v(v) {}
    void lower(detail::lowering& L) const {
        xtg_value imm;
        if (std::is_floating_point<T>::value) imm.f = (double)m_v;
        else if (std::is_unsigned<T>::value) imm.u = (uint64_t)m_v;
        else imm.i = (int64_t)m_v;
        L.node(XTG_OP_SCALAR, detail::dtype_of<T>::value, 0, 0, imm);
    }
    bool refers_to(const void*) const { return false; }
    std::size_t dimension() const { return 0; }

private:
    T m_v;
};

// closure: lvalue containers by reference, everything else by value
template <class E> struct closure { using type = std::conditional_t<std::is_lvalue_reference<E>::value, const std::decay_t<E>&, std::decay_t<E>>; };
template <class E> using closure_t = typename closure<E>::type;

template <class T, bool = is_xexpression<T>::value> struct wrap_scalar { using type = T; };
template <class T> struct wrap_scalar<T, false> { using type = xscalar<std::decay_t<T>>; };

template <class T> class element_ref;
template <class T> struct scalar_of { using type = T; };
template <class T> struct scalar_of<element_ref<T>> { using type = T; };
template <class T> using scalar_t = typename scalar_of<std::decay_t<T>>::type;

template <class E> decltype(auto) as_expression(E&& e, std::true_type) { return std::forward<E>(e); }
template <class E> auto as_expression(E&& e, std::false_type) { return xscalar<scalar_t<E>>((scalar_t<E>)e); }
template <class E> decltype(auto) as_expression(E&& e) {
    return as_expression(std::forward<E>(e), typename is_xexpression<E>::type());
}
template <class E> using expr_closure_t = std::conditional_t<is_xexpression<E>::value, closure_t<E>, xscalar<scalar_t<E>>>;

// functors: opcode + the value type the reference's functor returns
namespace detail {
struct op_plus { static constexpr int code = XTG_OP_ADD; template <class A, class B> static auto t(A a, B b) -> decltype(a + b); };
struct op_minus { static constexpr int code = XTG_OP_SUB; template <class A, class B> static auto t(A a, B b) -> decltype(a - b); };
struct op_mul { static constexpr int code = XTG_OP_MUL; template <class A, class B> static auto t(A a, B b) -> decltype(a * b); };
struct op_div { static constexpr int code = XTG_OP_DIV; template <class A, class B> static auto t(A a, B b) -> decltype(a / b); };
struct op_mod { static constexpr int code = XTG_OP_MOD; template <class A, class B> static auto t(A a, B b) -> decltype(a % b); };
struct op_max { static constexpr int code = XTG_OP_MAXIMUM; template <class A, class B> static auto t(A a, B b) -> decltype(a > b ? a : b); };
struct op_min { static constexpr int code = XTG_OP_MINIMUM; template <class A, class B> static auto t(A a, B b) -> decltype(a < b ? a : b); };
struct op_lt { static constexpr int code = XTG_OP_LT; template <class A, class B> static bool t(A, B); };
struct op_le { static constexpr int code = XTG_OP_LE; template <class A, class B> static bool t(A, B); };
struct op_gt { static constexpr int code = XTG_OP_GT; template <class A, class B> static bool t(A, B); };
struct op_ge { static constexpr int code = XTG_OP_GE; template <class A, class B> static bool t(A, B); };
struct op_eq { static constexpr int code = XTG_OP_EQ; template <class A, class B> static bool t(A, B); };
struct op_ne { static constexpr int code = XTG_OP_NE; template <class A, class B> static bool t(A, B); };
struct op_and { static constexpr int code = XTG_OP_LOGICAL_AND; template <class A, class B> static bool t(A, B); };
struct op_or { static constexpr int code = XTG_OP_LOGICAL_OR; template <class A, class B> static bool t(A, B); };
struct op_pow { static constexpr int code = XTG_OP_POW; template <class A, class B> static auto t(A a, B b) -> decltype(std::pow(a, b)); };

struct op_neg { static constexpr int code = XTG_OP_NEG; template <class A> static auto t(A a) -> decltype(-a); };
struct op_exp { static constexpr int code = XTG_OP_EXP; template <class A> static auto t(A a) -> decltype(std::exp(a)); };
struct op_log { static constexpr int code = XTG_OP_LOG; template <class A> static auto t(A a) -> decltype(std::log(a)); };
struct op_sqrt { static constexpr int code = XTG_OP_SQRT; template <class A> static auto t(A a) -> decltype(std::sqrt(a)); };
struct op_abs { static constexpr int code = XTG_OP_ABS; template <class A> static auto t(A a) -> decltype(std::abs(a)); };
struct op_square { static constexpr int code = XTG_OP_SQUARE; template <class A> static auto t(A a) -> decltype(a * a); };
struct op_sin { static constexpr int code = XTG_OP_SIN; template <class A> static auto t(A a) -> decltype(std::sin(a)); };
struct op_cos { static constexpr int code = XTG_OP_COS; template <class A> static auto t(A a) -> decltype(std::cos(a)); };
struct op_tanh { static constexpr int code = XTG_OP_TANH; template <class A> static auto t(A a) -> decltype(std::tanh(a)); };
struct op_not { static constexpr int code = XTG_OP_LOGICAL_NOT; template <class A> static bool t(A); };
}  // namespace detail

template <class T> inline const void* id_of(const T& x) { return (const void*)&x; }

// n-ary lazy node (the lowered form of xfunction<F, CT...>)
template <class F, class... CT> class xfunction : public xexpression<xfunction<F, CT...>> {
public:
    using value_type = decltype(F::t(std::declval<typename std::decay_t<CT>::value_type>()...));
    template <class... A> explicit xfunction(A&&... a) : m_args(std::forward<A>(a)...) {}
    void lower(detail::lowering& L) const {
        lower_args(L, std::index_sequence_for<CT...>());
        L.node(F::code, detail::dtype_of<value_type>::value);
    }
    bool refers_to(const void* p) const { return refers(p, std::index_sequence_for<CT...>()); }
    std::size_t dimension() const { return dim(std::index_sequence_for<CT...>()); }
    const std::tuple<CT...>& args() const { return m_args; }

private:
    template <std::size_t... I> void lower_args(detail::lowering& L, std::index_sequence<I...>) const {
        (void)std::initializer_list<int>{(std::get<I>(m_args).lower(L), 0)...};
    }
    template <std::size_t... I> bool refers(const void* p, std::index_sequence<I...>) const {
        bool r = false;
        (void)std::initializer_list<int>{(r = r || std::get<I>(m_args).refers_to(p), 0)...};
        return r;
    }
    template <std::size_t... I> std::size_t dim(std::index_sequence<I...>) const {
        std::size_t d = 0;
        (void)std::initializer_list<int>{(d = std::max(d, std::get<I>(m_args).dimension()), 0)...};
        return d;
    }
    std::tuple<CT...> m_args;
};

template <class F, class... E> auto make_xfunction(E&&... e) {
    return xfunction<F, expr_closure_t<E>...>(as_expression(std::forward<E>(e))...);
}

// where(cond, a, b) — conditional_ternary (xoperation.hpp:127-143)
template <class C, class A, class B> class xwhere : public xexpression<xwhere<C, A, B>> {
public:
    using value_type = std::common_type_t<typename std::decay_t<A>::value_type, typename std::decay_t<B>::value_type>;
    template <class X, class Y, class Z> xwhere(X&& c, Y&& a, Z&& b) : m_c(std::forward<X>(c)), m_a(std::forward<Y>(a)), m_b(std::forward<Z>(b)) {}
    void lower(detail::lowering& L) const {
        m_c.lower(L);
        m_a.lower(L);
        m_b.lower(L);
        L.node(XTG_OP_WHERE, detail::dtype_of<value_type>::value);
    }
    bool refers_to(const void* p) const { return m_c.refers_to(p) || m_a.refers_to(p) || m_b.refers_to(p); }
    std::size_t dimension() const { return std::max({m_c.dimension(), m_a.dimension(), m_b.dimension()}); }

private:
    C m_c;
    A m_a;
    B m_b;
};

// cast<T>(e)
template <class T, class E> class xcast : public xexpression<xcast<T, E>> {
public:
    using value_type = T;
    template <class X> explicit xcast(X&& e) : m_e(std::forward<X>(e)) {}
    void lower(detail::lowering& L) const {
        m_e.lower(L);
        L.node(XTG_OP_CAST, detail::dtype_of<T>::value, detail::dtype_of<T>::value);
    }
    bool refers_to(const void* p) const { return m_e.refers_to(p); }
    std::size_t dimension() const { return m_e.dimension(); }

private:
    E m_e;
};

#define XTG_XT_BINARY(OPNAME, FUNCTOR)                                                                   \
    template <class E1, class E2, std::enable_if_t<is_xexpression<E1>::value || is_xexpression<E2>::value, int> = 0> \
    inline auto OPNAME(E1&& e1, E2&& e2) {                                                               \
        return make_xfunction<detail::FUNCTOR>(std::forward<E1>(e1), std::forward<E2>(e2));              \
    }
XTG_XT_BINARY(operator+, op_plus)
XTG_XT_BINARY(operator-, op_minus)
XTG_XT_BINARY(operator*, op_mul)
XTG_XT_BINARY(operator/, op_div)
XTG_XT_BINARY(operator%, op_mod)
XTG_XT_BINARY(operator<, op_lt)
XTG_XT_BINARY(operator<=, op_le)
XTG_XT_BINARY(operator>, op_gt)
XTG_XT_BINARY(operator>=, op_ge)
XTG_XT_BINARY(operator&&, op_and)
XTG_XT_BINARY(operator||, op_or)
XTG_XT_BINARY(maximum, op_max)
XTG_XT_BINARY(minimum, op_min)
XTG_XT_BINARY(pow, op_pow)
XTG_XT_BINARY(equal, op_eq)
XTG_XT_BINARY(not_equal, op_ne)
#undef XTG_XT_BINARY

#define XTG_XT_UNARY(OPNAME, FUNCTOR)                                                          \
    template <class E, std::enable_if_t<is_xexpression<E>::value, int> = 0>                   \
    inline auto OPNAME(E&& e) {                                                                \
        return make_xfunction<detail::FUNCTOR>(std::forward<E>(e));                            \
    }
XTG_XT_UNARY(operator-, op_neg)
XTG_XT_UNARY(operator!, op_not)
XTG_XT_UNARY(exp, op_exp)
XTG_XT_UNARY(log, op_log)
XTG_XT_UNARY(sqrt, op_sqrt)
XTG_XT_UNARY(abs, op_abs)
XTG_XT_UNARY(fabs, op_abs)
XTG_XT_UNARY(square, op_square)
XTG_XT_UNARY(sin, op_sin)
XTG_XT_UNARY(cos, op_cos)
XTG_XT_UNARY(tanh, op_tanh)
#undef XTG_XT_UNARY

template <class C, class A, class B> inline auto where(C&& c, A&& a, B&& b) {
    return xwhere<expr_closure_t<C>, expr_closure_t<A>, expr_closure_t<B>>(
        as_expression(std::forward<C>(c)), as_expression(std::forward<A>(a)), as_expression(std::forward<B>(b)));
}
template <class T, class E> inline auto cast(E&& e) { return xcast<T, expr_closure_t<E>>(as_expression(std::forward<E>(e))); }

// ---------------------------------------------------------------------------- containers
namespace detail {
struct device_buffer {
    void* ptr = nullptr;
    std::size_t bytes = 0;
    std::shared_ptr<device_buffer> base;  // set: a view of `bytes` at `ptr` inside base (freed with it)
    explicit device_buffer(std::size_t b) : bytes(b) { check(xtg_malloc(&ptr, b ? b : 1, current_stream())); }
    device_buffer(std::shared_ptr<device_buffer> b, std::size_t offset, std::size_t n)
        : ptr((char*)b->ptr + offset), bytes(n), base(std::move(b)) {}
    ~device_buffer() {
        if (ptr && !base) xtg_free(ptr, current_stream());
    }
    device_buffer(const device_buffer&) = delete;
    device_buffer& operator=(const device_buffer&) = delete;
};
// tag of the constructor that adopts existing device storage
struct adopt_t {};
constexpr adopt_t adopt{};

template <class S> std::vector<std::ptrdiff_t> row_major_strides(const S& shape) {
    std::vector<std::ptrdiff_t> st(shape.size());
    std::ptrdiff_t acc = 1;
    for (std::size_t i = shape.size(); i-- > 0;) {
        st[i] = shape[i] == 1 ? 0 : acc;  // size-1 dims get stride 0 (xstrides.hpp:570-581)
        acc *= (std::ptrdiff_t)std::max<std::size_t>(shape[i], 1);
    }
    return st;
}

// nested initializer lists -> shape + flat data
template <class T> struct nested;
template <class T> struct nested {
    static void shape(const T&, std::vector<std::size_t>&, std::size_t) {}
    static void flat(const T& v, std::vector<T>& out) { out.push_back(v); }
};
template <class T> struct nested<std::initializer_list<T>> {
    static void shape(const std::initializer_list<T>& l, std::vector<std::size_t>& s, std::size_t d) {
        if (s.size() <= d) s.push_back(l.size());
        if (l.size()) nested<T>::shape(*l.begin(), s, d + 1);
    }
    template <class V> static void flat(const std::initializer_list<T>& l, std::vector<V>& out) {
        for (const auto& x : l) nested<T>::flat(x, out);
    }
};
}  // namespace detail

template <class T> class element_ref;

template <class T, std::ptrdiff_t N> class xdevice_container;
template <class T> using xarray = xdevice_container<T, -1>;
template <class T, std::size_t N> using xtensor = xdevice_container<T, (std::ptrdiff_t)N>;

template <class E> struct has_value_type_of;

template <class T, std::ptrdiff_t N>
class xdevice_container : public xexpression<xdevice_container<T, N>> {
public:
    using value_type = T;
    using size_type = std::size_t;
    using shape_type = std::conditional_t<(N < 0), std::vector<std::size_t>, std::array<std::size_t, (N < 0 ? 0 : N)>>;
    using strides_type = std::vector<std::ptrdiff_t>;

    xdevice_container() { set_shape(default_shape()); }
    template <class S, std::enable_if_t<!is_xexpression<S>::value && !std::is_arithmetic<S>::value, int> = 0>
    explicit xdevice_container(const S& shape) { set_shape(to_shape(shape)); }
    xdevice_container(const shape_type& shape, T fill_value) {
        set_shape(shape);
        fill(fill_value);
    }
    // 0-d from a scalar (xarray<double> b(1.2))
    template <class V, std::enable_if_t<std::is_arithmetic<V>::value && N <= 0, int> = 0>
    xdevice_container(V v) {
        set_shape(shape_type{});
        fill((T)v);
    }
    // nested initializer lists; a fixed-rank xtensor only takes its own depth
    template <std::ptrdiff_t M = N, std::enable_if_t<(M < 0 || M == 1), int> = 0>
    xdevice_container(std::initializer_list<T> l) { from_nested(l); }
    template <std::ptrdiff_t M = N, std::enable_if_t<(M < 0 || M == 2), int> = 0>
    xdevice_container(std::initializer_list<std::initializer_list<T>> l) { from_nested(l); }
    template <std::ptrdiff_t M = N, std::enable_if_t<(M < 0 || M == 3), int> = 0>
    xdevice_container(std::initializer_list<std::initializer_list<std::initializer_list<T>>> l) { from_nested(l); }
    template <std::ptrdiff_t M = N, std::enable_if_t<(M < 0 || M == 4), int> = 0>
    xdevice_container(std::initializer_list<std::initializer_list<std::initializer_list<std::initializer_list<T>>>> l) {
        from_nested(l);
    }
    template <class E> xdevice_container(const xexpression<E>& e) { assign_expr(e.derived_cast(), true); }
    // a row-major container of `shape` over existing device storage
    template <class S> xdevice_container(detail::adopt_t, const S& shape, std::shared_ptr<detail::device_buffer> buf) {
        set_shape(to_shape(shape), false);
        m_buf = std::move(buf);
    }
    xdevice_container(const xdevice_container& o) {
        set_shape(o.m_shape);
        copy_from(o);
    }
    xdevice_container(xdevice_container&&) noexcept = default;
    template <class U, std::ptrdiff_t M> xdevice_container(const xdevice_container<U, M>& o) { assign_expr(o, true); }

    xdevice_container& operator=(const xdevice_container& o) {
        if (this != &o) {
            set_shape(o.m_shape);
            copy_from(o);
        }
        return *this;
    }
    xdevice_container& operator=(xdevice_container&&) noexcept = default;
    template <class E> xdevice_container& operator=(const xexpression<E>& e) {
        assign_expr(e.derived_cast(), true);
        return *this;
    }
    xdevice_container& operator=(T v) {
        fill(v);
        return *this;
    }
    template <class E> xdevice_container& operator+=(const E& e) { return computed(*this + e); }
    template <class E> xdevice_container& operator-=(const E& e) { return computed(*this - e); }
    template <class E> xdevice_container& operator*=(const E& e) { return computed(*this * e); }
    template <class E> xdevice_container& operator/=(const E& e) { return computed(*this / e); }

    template <class S> static xdevice_container from_shape(const S& s) { return xdevice_container(s); }

    // geometry
    const shape_type& shape() const noexcept { return m_shape; }
    std::size_t shape(std::size_t i) const { return m_shape[i]; }
    const strides_type& strides() const noexcept { return m_strides; }
    std::size_t dimension() const noexcept { return m_shape.size(); }
    std::size_t size() const noexcept { return m_size; }
    T* data() noexcept { return m_buf ? (T*)m_buf->ptr : nullptr; }
    const T* data() const noexcept { return m_buf ? (const T*)m_buf->ptr : nullptr; }
    template <class S> void resize(const S& s) {
        auto ns = to_shape(s);
        // a container built from an expression has no storage yet, even when
        // its (default, 0-d) shape already matches
        if (!m_buf ||
            std::vector<std::size_t>(ns.begin(), ns.end()) != std::vector<std::size_t>(m_shape.begin(), m_shape.end()))
            set_shape(ns);
    }
    // in place; returns the container so that call sites can chain it
    // (`arange(1000).reshape({10, 10, 10})`)
    template <class S> xdevice_container& reshape(const S& s) {
        auto ns = to_shape(s);
        std::size_t n = 1;
        for (auto v : ns) n *= v;
        if (n != m_size) throw std::runtime_error("Cannot reshape with incorrect number of elements.");
        auto keep = m_buf;
        set_shape(ns, false);
        m_buf = keep;
        return *this;
    }
    template <class I> xdevice_container& reshape(std::initializer_list<I> s) {
        return reshape(std::vector<std::size_t>(s.begin(), s.end()));
    }
    void fill(T v) {
        std::vector<T> h(m_size, v);
        upload(h);
    }

    // element access: the trailing dims take the indices (xtensor's rule for
    // fewer indices than dimensions; extra leading indices are dropped)
    template <class... I> element_ref<T> operator()(I... idx) { return element_ref<T>(data() + offset(idx...)); }
    template <class... I> T operator()(I... idx) const { return element_ref<T>(const_cast<T*>(data()) + offset(idx...)); }
    template <class S> element_ref<T> element(const S& idx) { return element_ref<T>(data() + offset_seq(idx)); }
    element_ref<T> operator[](std::size_t i) { return element_ref<T>(data() + offset(i)); }
    T flat(std::size_t i) const { return element_ref<T>(const_cast<T*>(data()) + i); }

    // lowering as a leaf
    xtg_array xtg_desc() const {
        xtg_array a;
        std::memset(&a, 0, sizeof a);
        a.data = const_cast<T*>(data());
        a.dtype = detail::dtype_of<T>::value;
        a.rank = (int32_t)m_shape.size();
        for (std::size_t i = 0; i < m_shape.size(); ++i) {
            a.shape[i] = (int64_t)m_shape[i];
            a.strides[i] = (int64_t)m_strides[i];
        }
        return a;
    }
    void lower(detail::lowering& L) const {
        int i = L.leaf(xtg_desc(), this);
        L.node(XTG_OP_LEAF, detail::dtype_of<T>::value, i);
    }
    bool refers_to(const void* p) const { return p == (const void*)data(); }

    // host copies
    std::vector<T> to_host() const {
        if constexpr (std::is_same<T, bool>::value) {  // std::vector<bool> packs bits: go through bytes
            std::vector<unsigned char> b(m_size);
            if (m_size) {
                detail::check(xtg_memcpy(b.data(), data(), m_size, XTG_MEMCPY_D2H, detail::current_stream()));
                detail::check(xtg_stream_sync(detail::current_stream()));
            }
            return std::vector<bool>(b.begin(), b.end());
        } else {
            std::vector<T> h(m_size);
            if (m_size) {
                detail::check(xtg_memcpy(h.data(), data(), m_size * sizeof(T), XTG_MEMCPY_D2H, detail::current_stream()));
                detail::check(xtg_stream_sync(detail::current_stream()));
            }
            return h;
        }
    }
    void upload(const std::vector<T>& h) {
        if (!m_size) return;
        if constexpr (std::is_same<T, bool>::value) {
            std::vector<unsigned char> b(h.begin(), h.end());
            detail::check(xtg_memcpy(data(), b.data(), m_size, XTG_MEMCPY_H2D, detail::current_stream()));
        } else {
            detail::check(xtg_memcpy(data(), h.data(), m_size * sizeof(T), XTG_MEMCPY_H2D, detail::current_stream()));
        }
        detail::check(xtg_stream_sync(detail::current_stream()));
    }

    // evaluation entry points used by the free functions
    template <class E> void assign_expr(const E& e, bool may_alias);
    template <class E> void noalias_assign(const E& e);

private:
    static shape_type default_shape() {
        shape_type s{};
        if constexpr (N > 0)
            for (auto& v : s) v = 1;
        return s;
    }
    template <class S> static shape_type to_shape(const S& s) {
        shape_type r{};
        if constexpr (N < 0) {
            r.assign(std::begin(s), std::end(s));
        } else {
            if ((std::ptrdiff_t)std::distance(std::begin(s), std::end(s)) != N)
                throw std::runtime_error("xt: shape rank does not match xtensor rank");
            std::size_t i = 0;
            for (auto v : s) r[i++] = (std::size_t)v;
        }
        return r;
    }
    void set_shape(const shape_type& s, bool alloc = true) {
        m_shape = s;
        m_strides = detail::row_major_strides(s);
        m_size = 1;
        for (auto v : s) m_size *= v;
        if (alloc) m_buf = std::make_shared<detail::device_buffer>(m_size * sizeof(T));
    }
    template <class L> void from_nested(const L& l) {
        std::vector<std::size_t> s;
        detail::nested<L>::shape(l, s, 0);
        std::vector<T> h;
        detail::nested<L>::flat(l, h);
        set_shape(to_shape(s));
        upload(h);
    }
    void copy_from(const xdevice_container& o) {
        if (m_size)
            detail::check(xtg_memcpy(data(), o.data(), m_size * sizeof(T), XTG_MEMCPY_D2D, detail::current_stream()));
    }
    template <class E> xdevice_container& computed(const E& e) {
        noalias_assign(e);  // element-for-element aliasing is safe
        return *this;
    }
    template <class... I> std::size_t offset(I... idx) const {
        const std::ptrdiff_t v[] = {(std::ptrdiff_t)idx..., 0};
        const std::size_t n = sizeof...(I), r = m_shape.size();
        std::size_t o = 0;
        for (std::size_t k = 0; k < std::min(n, r); ++k) {
            const std::size_t d = r - std::min(n, r) + k;
            const std::ptrdiff_t i = v[n - std::min(n, r) + k];
            if (i < 0 || (std::size_t)i >= m_shape[d]) throw std::out_of_range("xt: index out of bounds");
            o += (std::size_t)(i * (m_shape[d] == 1 ? 0 : m_strides[d]));
        }
        return o;
    }
    template <class S> std::size_t offset_seq(const S& idx) const {
        std::size_t o = 0, d = 0;
        for (auto i : idx) o += (std::size_t)((std::ptrdiff_t)i * m_strides[d++]);
        return o;
    }

    shape_type m_shape{};
    strides_type m_strides;
    std::size_t m_size = 1;
    std::shared_ptr<detail::device_buffer> m_buf;
};

// an element of a device array: reads and writes copy one value
template <class T> class element_ref {
public:
    explicit element_ref(T* p) : m_p(p) {}
    operator T() const {
        T v{};
        detail::check(xtg_stream_sync(detail::current_stream()));
        detail::check(xtg_memcpy(&v, m_p, sizeof(T), XTG_MEMCPY_D2H, detail::current_stream()));
        detail::check(xtg_stream_sync(detail::current_stream()));
        return v;
    }
    element_ref& operator=(T v) {
        detail::check(xtg_memcpy(m_p, &v, sizeof(T), XTG_MEMCPY_H2D, detail::current_stream()));
        detail::check(xtg_stream_sync(detail::current_stream()));
        return *this;
    }
    element_ref& operator=(const element_ref& o) { return *this = (T)o; }

private:
    T* m_p;
};
template <class T> bool operator==(const element_ref<T>& a, const T& b) { return (T)a == b; }

// ---------------------------------------------------------------------------- strided views
template <class T> class xstrided_view : public xexpression<xstrided_view<T>> {
public:
    using value_type = T;
    xstrided_view(T* data, std::vector<std::size_t> shape, std::vector<std::ptrdiff_t> strides, std::shared_ptr<void> keep)
        : m_data(data), m_shape(std::move(shape)), m_strides(std::move(strides)), m_keep(std::move(keep)) {}
    const std::vector<std::size_t>& shape() const { return m_shape; }
    std::size_t dimension() const { return m_shape.size(); }
    std::size_t size() const {
        std::size_t n = 1;
        for (auto v : m_shape) n *= v;
        return n;
    }
    xtg_array xtg_desc() const {
        xtg_array a;
        std::memset(&a, 0, sizeof a);
        a.data = m_data;
        a.dtype = detail::dtype_of<T>::value;
        a.rank = (int32_t)m_shape.size();
        for (std::size_t i = 0; i < m_shape.size(); ++i) {
            a.shape[i] = (int64_t)m_shape[i];
            a.strides[i] = (int64_t)m_strides[i];
        }
        return a;
    }
    void lower(detail::lowering& L) const {
        int i = L.leaf(xtg_desc(), this);
        L.node(XTG_OP_LEAF, detail::dtype_of<T>::value, i);
    }
    bool refers_to(const void* p) const { return p == (const void*)m_base_hint(); }
    template <class E> xstrided_view& operator=(const xexpression<E>& e);
    xstrided_view& operator=(T v);

private:
    const void* m_base_hint() const { return m_data; }
    T* m_data;
    std::vector<std::size_t> m_shape;
    std::vector<std::ptrdiff_t> m_strides;
    std::shared_ptr<void> m_keep;
};

template <class T, std::ptrdiff_t N, class P>
inline auto transpose(xdevice_container<T, N>& a, const P& perm_in) {
    std::vector<std::size_t> perm(std::begin(perm_in), std::end(perm_in));
    if (perm.size() != a.dimension()) throw std::runtime_error("Permutation does not have the same size as shape");
    std::vector<std::size_t> s;
    std::vector<std::ptrdiff_t> st;
    for (auto p : perm) {
        s.push_back(a.shape()[p]);
        st.push_back(a.strides()[p]);
    }
    return xstrided_view<T>(a.data(), s, st, nullptr);
}
template <class T, std::ptrdiff_t N>
inline auto transpose(xdevice_container<T, N>& a, std::initializer_list<std::size_t> perm) {
    return transpose(a, std::vector<std::size_t>(perm));
}
template <class T, std::ptrdiff_t N> inline auto transpose(xdevice_container<T, N>& a) {
    std::vector<std::size_t> perm(a.dimension());
    for (std::size_t i = 0; i < perm.size(); ++i) perm[i] = perm.size() - 1 - i;
    return transpose(a, perm);
}

// xt::view slices: range(start, stop[, step]), all(), an integer index, newaxis()
struct xrange {
    std::ptrdiff_t start, stop, step;
};
struct xall_tag {};
struct xnewaxis_tag {};
inline xrange range(std::ptrdiff_t a, std::ptrdiff_t b, std::ptrdiff_t s = 1) { return {a, b, s}; }
inline xall_tag all() { return {}; }
inline xnewaxis_tag newaxis() { return {}; }

namespace detail {
struct view_builder {
    std::vector<std::size_t> shape;
    std::vector<std::ptrdiff_t> strides;
    std::ptrdiff_t offset = 0;
    std::size_t dim = 0;
    const std::vector<std::size_t>* src_shape;
    const std::vector<std::ptrdiff_t>* src_strides;
    void add(const xrange& r) {
        const std::ptrdiff_t n = (std::ptrdiff_t)(*src_shape)[dim];
        std::ptrdiff_t a = r.start < 0 ? r.start + n : r.start, b = r.stop < 0 ? r.stop + n : r.stop;
        a = std::max<std::ptrdiff_t>(0, std::min(a, n));
        b = std::max<std::ptrdiff_t>(0, std::min(b, n));
        const std::ptrdiff_t cnt = r.step > 0 ? std::max<std::ptrdiff_t>(0, (b - a + r.step - 1) / r.step) : 0;
        offset += a * (*src_strides)[dim];
        shape.push_back((std::size_t)cnt);
        strides.push_back((*src_strides)[dim] * r.step);
        ++dim;
    }
    void add(xall_tag) {
        shape.push_back((*src_shape)[dim]);
        strides.push_back((*src_strides)[dim]);
        ++dim;
    }
    void add(xnewaxis_tag) {
        shape.push_back(1);
        strides.push_back(0);
    }
    template <class I, std::enable_if_t<std::is_integral<I>::value, int> = 0> void add(I i) {
        std::ptrdiff_t k = (std::ptrdiff_t)i;
        if (k < 0) k += (std::ptrdiff_t)(*src_shape)[dim];
        offset += k * (*src_strides)[dim];
        ++dim;
    }
};
}  // namespace detail

template <class T, std::ptrdiff_t N, class... S> inline auto view(xdevice_container<T, N>& a, S... s) {
    std::vector<std::size_t> ss(a.shape().begin(), a.shape().end());
    std::vector<std::ptrdiff_t> st(a.strides().begin(), a.strides().end());
    for (std::size_t d = 0; d < ss.size(); ++d)
        if (ss[d] != 1 && st[d] == 0) st[d] = 0;
    // recompute dense strides (containers store 0 for size-1 dims)
    std::ptrdiff_t acc = 1;
    for (std::size_t d = ss.size(); d-- > 0;) {
        st[d] = acc;
        acc *= (std::ptrdiff_t)std::max<std::size_t>(ss[d], 1);
    }
    detail::view_builder b;
    b.src_shape = &ss;
    b.src_strides = &st;
    (void)std::initializer_list<int>{(b.add(s), 0)...};
    for (std::size_t d = b.dim; d < ss.size(); ++d) {
        b.shape.push_back(ss[d]);
        b.strides.push_back(st[d]);
    }
    return xstrided_view<T>(a.data() + b.offset, b.shape, b.strides, nullptr);
}

// ---------------------------------------------------------------------------- reducers
struct reducer_options {
    bool keep_dims = false;
    bool immediate = false;
    bool has_initial = false;
    double initial_f = 0;  // xt::initial(v), converted to the result type when used
    int64_t initial_i = 0;
};
inline reducer_options operator|(reducer_options a, const reducer_options& b) {
    a.keep_dims |= b.keep_dims;
    a.immediate |= b.immediate;
    if (b.has_initial) {
        a.has_initial = true;
        a.initial_f = b.initial_f;
        a.initial_i = b.initial_i;
    }
    return a;
}
struct keep_dims_type : reducer_options {
    keep_dims_type() { keep_dims = true; }
};
static const keep_dims_type keep_dims{};
namespace evaluation_strategy {
struct lazy_type : reducer_options {};
struct immediate_type : reducer_options {
    immediate_type() { immediate = true; }
};
static const lazy_type lazy{};
static const immediate_type immediate{};
}  // namespace evaluation_strategy
template <class V> inline reducer_options initial(V v) {
    reducer_options o;
    o.has_initial = true;
    o.initial_f = (double)v;
    o.initial_i = (int64_t)v;
    return o;
}

namespace detail {
template <class V> struct big_promote {
    using type = std::conditional_t<std::is_floating_point<V>::value, double,
                                    std::conditional_t<std::is_signed<V>::value, long long, unsigned long long>>;
};
template <int OP, class V, class T> struct red_result {
    using init = std::conditional_t<std::is_same<T, void>::value, V, T>;
    using type = decltype(std::declval<init>() + std::declval<V>());
};
template <class V, class T> struct red_result<XTG_RED_PROD, V, T> {
    using init = std::conditional_t<std::is_same<T, void>::value, V, T>;
    using type = decltype(std::declval<init>() * std::declval<V>());
};
template <class V, class T> struct red_result<XTG_RED_AMAX, V, T> { using type = std::common_type_t<T, V>; };
template <class V> struct red_result<XTG_RED_AMAX, V, void> { using type = V; };
template <class V, class T> struct red_result<XTG_RED_AMIN, V, T> : red_result<XTG_RED_AMAX, V, T> {};
template <class V, class T> struct red_result<XTG_RED_MEAN, V, T> {
    using type = std::conditional_t<std::is_same<T, void>::value, double, T>;
};
template <class V, class T> struct red_result<XTG_RED_VARIANCE, V, T> : red_result<XTG_RED_MEAN, V, T> {};
template <class V, class T> struct red_result<XTG_RED_STDDEV, V, T> : red_result<XTG_RED_MEAN, V, T> {};
template <class V, class T> struct red_result<XTG_RED_NORM_L0, V, T> { using type = unsigned long long; };
template <class V, class T> struct red_result<XTG_RED_NORM_L1, V, T> { using type = typename big_promote<V>::type; };
template <class V, class T> struct red_result<XTG_RED_NORM_SQ, V, T> { using type = typename big_promote<V>::type; };
template <class V, class T> struct red_result<XTG_RED_NORM_L2, V, T> { using type = double; };
template <class V, class T> struct red_result<XTG_RED_NORM_LINF, V, T> { using type = decltype(std::abs(std::declval<V>())); };
}  // namespace detail

template <int OP, class T, class E> class xreducer : public xexpression<xreducer<OP, T, E>> {
public:
    using value_type = typename detail::red_result<OP, typename std::decay_t<E>::value_type, T>::type;
    template <class X> xreducer(X&& e, std::vector<std::ptrdiff_t> axes, bool all_axes, reducer_options o, int64_t ddof = 0)
        : m_e(std::forward<X>(e)), m_axes(std::move(axes)), m_all(all_axes), m_o(o), m_ddof(ddof) {}
    xtg_reduce_desc desc() const {
        xtg_reduce_desc d;
        std::memset(&d, 0, sizeof d);
        d.op = OP;
        d.n_axes = m_all ? -1 : (int32_t)m_axes.size();
        for (std::size_t i = 0; i < m_axes.size() && i < XTG_MAX_RANK; ++i) d.axes[i] = m_axes[i];
        d.keep_dims = m_o.keep_dims;
        d.has_initial = m_o.has_initial;
        if (std::is_floating_point<value_type>::value) d.initial.f = m_o.initial_f;
        else d.initial.i = m_o.initial_i;
        d.acc_dtype = std::is_same<T, void>::value ? -1 : detail::dtype_of<std::conditional_t<std::is_same<T, void>::value, int, T>>::value;
        d.precision = XTG_PREC_COMPENSATED;
        d.ddof = m_ddof;
        return d;
    }
    std::vector<std::size_t> shape() const {
        detail::lowering L;
        m_e.lower(L);
        xtg_reduce_desc d = desc();
        int32_t r = 0, dt = 0;
        int64_t sh[XTG_MAX_RANK];
        detail::check(xtg_reduce_shape(&L.e, &d, &r, sh, &dt));
        return std::vector<std::size_t>(sh, sh + r);
    }
    std::size_t dimension() const { return shape().size(); }
    // evaluates into `out` (already shaped)
    template <class C> void evaluate_into(C& out) const {
        detail::lowering L;
        m_e.lower(L);
        xtg_reduce_desc d = desc();
        xtg_array o = out.xtg_desc();
        if (const xtg_chunked* c = L.only_chunked()) {
            if (!d.has_initial && d.ddof == 0 && d.acc_dtype < 0) {
                detail::check(xtg_chunked_reduce(c, &d, &o, detail::current_stream()));
                return;
            }
        }
        detail::resolve_chunked(L);
        detail::check(xtg_reduce(&L.e, &d, &o, detail::current_stream()));
    }
    xarray<value_type> eval() const {
        xarray<value_type> out(shape());
        evaluate_into(out);
        return out;
    }
    template <class... I> value_type operator()(I... idx) const { return eval()(idx...); }
    value_type operator()() const {
        auto r = eval();
        return r.flat(0);
    }
    value_type operator[](std::size_t i) const { return eval().flat(i); }
    // as an operand: keep-dims trailing-axis statistics lower to row nodes,
    // everything else is evaluated into a temporary leaf
    void lower(detail::lowering& L) const {
        const std::size_t nd = m_e.dimension();
        bool trailing = m_o.keep_dims && !m_all && !m_axes.empty() && !m_o.has_initial;
        for (std::size_t i = 0; trailing && i < m_axes.size(); ++i) {
            std::ptrdiff_t a = m_axes[i] < 0 ? m_axes[i] + (std::ptrdiff_t)nd : m_axes[i];
            if (a != (std::ptrdiff_t)(nd - m_axes.size() + i)) trailing = false;
        }
        const int rop = OP == XTG_RED_SUM ? XTG_OP_RSUM : OP == XTG_RED_MEAN ? XTG_OP_RMEAN : OP == XTG_RED_VARIANCE ? XTG_OP_RVAR
                      : OP == XTG_RED_STDDEV ? XTG_OP_RSTD : OP == XTG_RED_AMAX ? XTG_OP_RMAX : OP == XTG_RED_AMIN ? XTG_OP_RMIN : -1;
        if (trailing && rop >= 0 && std::is_same<T, void>::value) {
            m_e.lower(L);
            L.node(rop, detail::dtype_of<value_type>::value, (int)m_axes.size(), (int)m_ddof);
            return;
        }
        auto tmp = std::make_shared<xarray<value_type>>(eval());
        L.temps.push_back(tmp);
        int i = L.leaf(tmp->xtg_desc(), tmp.get());
        L.node(XTG_OP_LEAF, detail::dtype_of<value_type>::value, i);
    }
    bool refers_to(const void* p) const { return m_e.refers_to(p); }

private:
    E m_e;
    std::vector<std::ptrdiff_t> m_axes;
    bool m_all;
    reducer_options m_o;
    int64_t m_ddof;
};

namespace detail {
template <class X> std::vector<std::ptrdiff_t> axes_vec(const X& x) {
    return std::vector<std::ptrdiff_t>(std::begin(x), std::end(x));
}
template <int OP, class T, class E> auto make_reducer(E&& e, std::vector<std::ptrdiff_t> axes, bool all, reducer_options o,
                                                     int64_t ddof = 0) {
    return xreducer<OP, T, closure_t<E>>(std::forward<E>(e), std::move(axes), all, o, ddof);
}
}  // namespace detail

#define XTG_XT_REDUCER(NAME, OP)                                                                                   \
    template <class T = void, class E, std::enable_if_t<is_xexpression<E>::value, int> = 0>                         \
    inline auto NAME(E&& e, reducer_options o = {}) {                                                              \
        return detail::make_reducer<OP, T>(std::forward<E>(e), {}, true, o);                                        \
    }                                                                                                              \
    template <class T = void, class E, class I, std::enable_if_t<std::is_integral<I>::value, int> = 0>              \
    inline auto NAME(E&& e, std::initializer_list<I> axes, reducer_options o = {}) {                               \
        return detail::make_reducer<OP, T>(std::forward<E>(e), detail::axes_vec(axes), false, o);                   \
    }                                                                                                              \
    template <class T = void, class E, class X,                                                                   \
              std::enable_if_t<!std::is_integral<std::decay_t<X>>::value && !std::is_base_of<reducer_options, std::decay_t<X>>::value, int> = 0> \
    inline auto NAME(E&& e, const X& axes, reducer_options o = {}) {                                               \
        return detail::make_reducer<OP, T>(std::forward<E>(e), detail::axes_vec(axes), false, o);                   \
    }                                                                                                              \
    template <class T = void, class E, class I, std::enable_if_t<std::is_integral<I>::value, int> = 0>              \
    inline auto NAME(E&& e, I axis, reducer_options o = {}) {                                                      \
        return detail::make_reducer<OP, T>(std::forward<E>(e), {(std::ptrdiff_t)axis}, false, o);                   \
    }
XTG_XT_REDUCER(sum, XTG_RED_SUM)
XTG_XT_REDUCER(prod, XTG_RED_PROD)
XTG_XT_REDUCER(amax, XTG_RED_AMAX)
XTG_XT_REDUCER(amin, XTG_RED_AMIN)
XTG_XT_REDUCER(mean, XTG_RED_MEAN)
XTG_XT_REDUCER(norm_l0, XTG_RED_NORM_L0)
XTG_XT_REDUCER(norm_l1, XTG_RED_NORM_L1)
XTG_XT_REDUCER(norm_sq, XTG_RED_NORM_SQ)
XTG_XT_REDUCER(norm_l2, XTG_RED_NORM_L2)
XTG_XT_REDUCER(norm_linf, XTG_RED_NORM_LINF)
#undef XTG_XT_REDUCER

// variance / stddev with ddof (xmath.hpp:2033-2180)
#define XTG_XT_MOMENT(NAME, OP)                                                                                    \
    template <class T = void, class E, std::enable_if_t<is_xexpression<E>::value, int> = 0>                         \
    inline auto NAME(E&& e, reducer_options o = {}) {                                                              \
        return detail::make_reducer<OP, T>(std::forward<E>(e), {}, true, o);                                        \
    }                                                                                                              \
    template <class T = void, class E, class I, std::enable_if_t<std::is_integral<I>::value, int> = 0>              \
    inline auto NAME(E&& e, std::initializer_list<I> axes, reducer_options o = {}) {                               \
        return detail::make_reducer<OP, T>(std::forward<E>(e), detail::axes_vec(axes), false, o);                   \
    }                                                                                                              \
    template <class T = void, class E, class I, class D,                                                           \
              std::enable_if_t<std::is_integral<I>::value && std::is_integral<D>::value, int> = 0>                  \
    inline auto NAME(E&& e, std::initializer_list<I> axes, D ddof, reducer_options o = {}) {                       \
        return detail::make_reducer<OP, T>(std::forward<E>(e), detail::axes_vec(axes), false, o, (int64_t)ddof);    \
    }                                                                                                              \
    template <class T = void, class E, class I, std::enable_if_t<std::is_integral<I>::value, int> = 0>              \
    inline auto NAME(E&& e, I axis, reducer_options o = {}) {                                                      \
        return detail::make_reducer<OP, T>(std::forward<E>(e), {(std::ptrdiff_t)axis}, false, o);                   \
    }                                                                                                              \
    template <class T = void, class E, class X,                                                                   \
              std::enable_if_t<!std::is_integral<std::decay_t<X>>::value && !std::is_base_of<reducer_options, std::decay_t<X>>::value, int> = 0> \
    inline auto NAME(E&& e, const X& axes, reducer_options o = {}) {                                               \
        return detail::make_reducer<OP, T>(std::forward<E>(e), detail::axes_vec(axes), false, o);                   \
    }                                                                                                              \
    template <class T = void, class E, class X, class D,                                                           \
              std::enable_if_t<!std::is_integral<std::decay_t<X>>::value && std::is_integral<D>::value, int> = 0>   \
    inline auto NAME(E&& e, const X& axes, D ddof, reducer_options o = {}) {                                       \
        return detail::make_reducer<OP, T>(std::forward<E>(e), detail::axes_vec(axes), false, o, (int64_t)ddof);    \
    }
XTG_XT_MOMENT(variance, XTG_RED_VARIANCE)
XTG_XT_MOMENT(stddev, XTG_RED_STDDEV)
#undef XTG_XT_MOMENT

// ---------------------------------------------------------------------------- assignment
namespace detail {
template <class E> std::vector<std::size_t> broadcast_shape_of(const E& e) {
    lowering L;
    e.lower(L);
    int32_t r = 0;
    int64_t sh[XTG_MAX_RANK];
    check(xtg_broadcast_shape(&L.e, &r, sh));
    return std::vector<std::size_t>(sh, sh + r);
}
template <class E> struct is_reducer : std::false_type {};
template <int OP, class T, class E> struct is_reducer<xreducer<OP, T, E>> : std::true_type {};
}  // namespace detail

template <class T, std::ptrdiff_t N>
template <class E>
void xdevice_container<T, N>::assign_expr(const E& e, bool may_alias) {
    if constexpr (detail::is_reducer<E>::value) {
        auto s = e.shape();
        if (may_alias && e.refers_to(data())) {
            xdevice_container tmp(s);
            e.evaluate_into(tmp);
            *this = std::move(tmp);
            return;
        }
        resize(s);
        e.evaluate_into(*this);
    } else {
        auto s = detail::broadcast_shape_of(e);
        if (may_alias && m_buf && e.refers_to(data())) {
            xdevice_container tmp(s);
            tmp.noalias_assign(e);
            *this = std::move(tmp);
            return;
        }
        resize(s);
        noalias_assign(e);
    }
}

template <class T, std::ptrdiff_t N>
template <class E>
void xdevice_container<T, N>::noalias_assign(const E& e) {
    if constexpr (detail::is_reducer<E>::value) {
        e.evaluate_into(*this);
    } else {
        detail::lowering L;
        e.lower(L);
        xtg_array o = xtg_desc();
        if (const xtg_chunked* c = L.only_chunked()) {  // reading a chunked array
            detail::check(xtg_chunked_to_dense(c, &o, detail::current_stream()));
            return;
        }
        detail::resolve_chunked(L);
        detail::check(xtg_assign(&L.e, &o, detail::current_stream()));
    }
}

template <class T> template <class E> xstrided_view<T>& xstrided_view<T>::operator=(const xexpression<E>& e) {
    detail::lowering L;
    e.derived_cast().lower(L);
    xtg_array o = xtg_desc();
    detail::resolve_chunked(L);
    detail::check(xtg_assign(&L.e, &o, detail::current_stream()));
    return *this;
}
template <class T> xstrided_view<T>& xstrided_view<T>::operator=(T v) {
    return *this = xscalar<T>(v);
}

// noalias(a) = e
template <class C> class noalias_proxy {
public:
    explicit noalias_proxy(C& c) : m_c(c) {}
    template <class E> C& operator=(const xexpression<E>& e) {
        if constexpr (!std::is_same<C, xstrided_view<typename C::value_type>>::value) {
            if constexpr (detail::is_reducer<E>::value) m_c.resize(e.derived_cast().shape());
            else m_c.resize(detail::broadcast_shape_of(e.derived_cast()));
            m_c.noalias_assign(e.derived_cast());
        } else {
            m_c = e;
        }
        return m_c;
    }
    template <class E> C& operator+=(const xexpression<E>& e) { return *this = m_c + e.derived_cast(); }
    template <class E> C& operator-=(const xexpression<E>& e) { return *this = m_c - e.derived_cast(); }
    template <class E> C& operator*=(const xexpression<E>& e) { return *this = m_c * e.derived_cast(); }

private:
    C& m_c;
};
template <class C> inline noalias_proxy<C> noalias(C& c) { return noalias_proxy<C>(c); }

template <class E, std::enable_if_t<is_xexpression<E>::value, int> = 0> inline auto eval(const E& e) {
    using V = typename std::decay_t<E>::value_type;
    return xarray<V>(e);
}
template <class T, std::ptrdiff_t N> inline const xdevice_container<T, N>& eval(const xdevice_container<T, N>& c) { return c; }

// ---------------------------------------------------------------------------- arg reductions
template <class E> inline xarray<std::size_t> argmax(const xexpression<E>& e) {
    detail::lowering L;
    e.derived_cast().lower(L);
    xarray<std::size_t> out(std::vector<std::size_t>{});
    xtg_array o = out.xtg_desc();
    detail::resolve_chunked(L);
    detail::check(xtg_argreduce(&L.e, XTG_ARGMAX, 0, 0, &o, detail::current_stream()));
    return out;
}
template <class E> inline xarray<std::size_t> argmin(const xexpression<E>& e) {
    detail::lowering L;
    e.derived_cast().lower(L);
    xarray<std::size_t> out(std::vector<std::size_t>{});
    xtg_array o = out.xtg_desc();
    detail::resolve_chunked(L);
    detail::check(xtg_argreduce(&L.e, XTG_ARGMIN, 0, 0, &o, detail::current_stream()));
    return out;
}
namespace detail {
template <class E> xarray<std::size_t> arg_axis(const E& e, std::ptrdiff_t axis, int op) {
    lowering L;
    e.lower(L);
    int32_t r = 0;
    int64_t sh[XTG_MAX_RANK];
    check(xtg_broadcast_shape(&L.e, &r, sh));
    std::vector<std::size_t> os;
    if (r > 1) {
        std::ptrdiff_t a = axis < 0 ? axis + r : axis;
        if (a < 0 || a >= r) throw std::out_of_range("Axis larger than the dimension");
        for (int d = 0; d < r; ++d)
            if (d != a) os.push_back((std::size_t)sh[d]);
    }
    xarray<std::size_t> out(os);
    xtg_array o = out.xtg_desc();
    resolve_chunked(L);
    check(xtg_argreduce(&L.e, op, 1, axis, &o, current_stream()));
    return out;
}
}  // namespace detail
template <class E> inline xarray<std::size_t> argmax(const xexpression<E>& e, std::ptrdiff_t axis) {
    return detail::arg_axis(e.derived_cast(), axis, XTG_ARGMAX);
}
template <class E> inline xarray<std::size_t> argmin(const xexpression<E>& e, std::ptrdiff_t axis) {
    return detail::arg_axis(e.derived_cast(), axis, XTG_ARGMIN);
}

// ---------------------------------------------------------------------------- accumulators
// xt::cumsum / cumprod / nancumsum / nancumprod (include/xtensor/core/xmath.hpp:
// 2248-2301, 2592-2645): eager, like the reference's immediate accumulators;
// the element type is decltype(T-or-value_type{} op value_type{}).
namespace detail {
template <class R, class E> xarray<R> accumulate_into(const E& e, int op, int has_axis, std::ptrdiff_t axis) {
    lowering L;
    e.lower(L);
    int32_t r = 0, dt = 0;
    int64_t sh[XTG_MAX_RANK];
    check(xtg_accumulate_shape(&L.e, op, has_axis, axis, dtype_of<R>::value, &r, sh, &dt));
    xarray<R> out(std::vector<std::size_t>(sh, sh + r));
    xtg_array o = out.xtg_desc();
    resolve_chunked(L);
    check(xtg_accumulate(&L.e, op, has_axis, axis, dtype_of<R>::value, &o, current_stream()));
    return out;
}
template <class T, class E, int PROD> struct acc_result {
    using V = typename std::decay_t<E>::value_type;
    using I = std::conditional_t<std::is_void<T>::value, V, T>;
    using type = std::conditional_t<PROD != 0, decltype(std::declval<I>() * std::declval<V>()),
                                    decltype(std::declval<I>() + std::declval<V>())>;
};
}  // namespace detail
#define XTG_ACCUMULATOR(NAME, CODE, PROD)                                                                     \
    template <class T = void, class E>                                                                         \
    inline auto NAME(const xexpression<E>& e, std::ptrdiff_t axis) {                                           \
        return detail::accumulate_into<typename detail::acc_result<T, E, PROD>::type>(e.derived_cast(), CODE, 1, axis); \
    }                                                                                                          \
    template <class T = void, class E>                                                                         \
    inline auto NAME(const xexpression<E>& e) {                                                                \
        return detail::accumulate_into<typename detail::acc_result<T, E, PROD>::type>(e.derived_cast(), CODE, 0, 0); \
    }
XTG_ACCUMULATOR(cumsum, XTG_ACC_CUMSUM, 0)
XTG_ACCUMULATOR(cumprod, XTG_ACC_CUMPROD, 1)
XTG_ACCUMULATOR(nancumsum, XTG_ACC_NANCUMSUM, 0)
XTG_ACCUMULATOR(nancumprod, XTG_ACC_NANCUMPROD, 1)
#undef XTG_ACCUMULATOR

// ---------------------------------------------------------------------------- blockwise reducers
// xt::blockwise::<op>(e, block_shape, axes, options)
// (include/xtensor/reducers/xblockwise_reducer.hpp:269-533): the reducer's
// shape(), dimension() and assign_to(result) as the reference's; the work is
// libxtg's slab-streamed blockwise reduction.  `e` is a device expression
// (evaluated first) or an xt::host_array<T> — a dense host buffer, possibly
// larger than device memory, streamed through in slabs of whole blocks.
template <class T> struct host_array {
    using value_type = T;
    const T* data;
    std::vector<std::size_t> shape;
    std::vector<std::ptrdiff_t> strides;
};
template <class T, class S> inline host_array<T> adapt_host(const T* data, const S& shape) {
    host_array<T> h{data, std::vector<std::size_t>(std::begin(shape), std::end(shape)), {}};
    h.strides = detail::row_major_strides(h.shape);
    return h;
}
template <class T> inline host_array<T> adapt_host(const T* data, std::initializer_list<std::size_t> shape) {
    return adapt_host(data, std::vector<std::size_t>(shape));
}

template <int OP, class R> class xblockwise_reducer {
public:
    using value_type = R;
    template <class E, class BS, class X>
    xblockwise_reducer(const E& e, const BS& block_shape, const X& axes, bool all_axes, reducer_options o, double p)
        : m_p(p) {
        bind(e);
        m_block.assign(std::begin(block_shape), std::end(block_shape));
        std::memset(&m_rd, 0, sizeof m_rd);
        m_rd.op = OP;
        m_rd.n_axes = all_axes ? -1 : 0;
        if (!all_axes)
            for (auto a : axes) m_rd.axes[m_rd.n_axes++] = (int64_t)a;
        m_rd.keep_dims = o.keep_dims;
        m_rd.has_initial = o.has_initial;
        m_rd.acc_dtype = detail::dtype_of<R>::value;
        if (OP == XTG_RED_AMAX || OP == XTG_RED_AMIN || OP >= XTG_RED_NORM_L0) m_rd.acc_dtype = -1;
        int32_t r = 0, dt = 0;
        int64_t sh[XTG_MAX_RANK];
        detail::check(xtg_blockwise_shape(&m_in, &m_rd, &r, sh, &dt));
        m_shape.assign(sh, sh + r);
    }
    const std::vector<std::size_t>& shape() const { return m_shape; }
    std::size_t dimension() const { return m_shape.size(); }
    template <class D> void assign_to(D& result) const {
        const xtg_array o = result.xtg_desc();
        detail::check(xtg_blockwise_reduce(&m_in, m_block.data(), &m_rd, m_p, &o, detail::current_stream()));
    }

private:
    template <class T> void bind(const host_array<T>& h) {
        std::memset(&m_in, 0, sizeof m_in);
        m_in.data = const_cast<T*>(h.data);
        m_in.dtype = detail::dtype_of<T>::value;
        m_in.rank = (int32_t)h.shape.size();
        for (std::size_t i = 0; i < h.shape.size(); ++i) {
            m_in.shape[i] = (int64_t)h.shape[i];
            m_in.strides[i] = (int64_t)h.strides[i];
        }
    }
    template <class E> void bind(const E& e) {
        using V = typename std::decay_t<E>::value_type;
        auto ev = std::make_shared<xarray<V>>(xt::eval(e));
        m_keep = ev;
        m_in = ev->xtg_desc();
    }
    xtg_array m_in;
    std::shared_ptr<void> m_keep;
    std::vector<int64_t> m_block;
    xtg_reduce_desc m_rd;
    double m_p;
    std::vector<std::size_t> m_shape;
};

namespace blockwise {
namespace detail {
template <class E> struct value_of { using type = typename std::decay_t<E>::value_type; };
}  // namespace detail
#define XTG_BLOCKWISE(NAME, CODE)                                                                                  \
    template <class T = void, class E, class BS, class X,                                                           \
              std::enable_if_t<!std::is_integral<X>::value && !std::is_base_of<reducer_options, X>::value, int> = 0> \
    inline auto NAME(const E& e, const BS& block_shape, const X& axes, reducer_options o = {}) {                    \
        using R = typename xt::detail::red_result<CODE, typename detail::value_of<E>::type, T>::type;              \
        return xblockwise_reducer<CODE, R>(e, block_shape, axes, false, o, 0.0);                                    \
    }                                                                                                               \
    template <class T = void, class E, class BS>                                                                    \
    inline auto NAME(const E& e, const BS& block_shape, std::initializer_list<std::size_t> axes,                    \
                     reducer_options o = {}) {                                                                      \
        return NAME<T>(e, block_shape, std::vector<std::size_t>(axes), o);                                          \
    }                                                                                                               \
    template <class T = void, class E, class BS, class I, std::enable_if_t<std::is_integral<I>::value, int> = 0>    \
    inline auto NAME(const E& e, const BS& block_shape, I axis, reducer_options o = {}) {                           \
        return NAME<T>(e, block_shape, std::vector<std::size_t>{(std::size_t)axis}, o);                             \
    }                                                                                                               \
    template <class T = void, class E, class BS>                                                                    \
    inline auto NAME(const E& e, const BS& block_shape, reducer_options o = {}) {                                   \
        using R = typename xt::detail::red_result<CODE, typename detail::value_of<E>::type, T>::type;              \
        return xblockwise_reducer<CODE, R>(e, block_shape, std::vector<std::size_t>{}, true, o, 0.0);               \
    }
XTG_BLOCKWISE(sum, XTG_RED_SUM)
XTG_BLOCKWISE(prod, XTG_RED_PROD)
XTG_BLOCKWISE(amin, XTG_RED_AMIN)
XTG_BLOCKWISE(amax, XTG_RED_AMAX)
XTG_BLOCKWISE(mean, XTG_RED_MEAN)
XTG_BLOCKWISE(variance, XTG_RED_VARIANCE)
XTG_BLOCKWISE(stddev, XTG_RED_STDDEV)
XTG_BLOCKWISE(norm_l0, XTG_RED_NORM_L0)
XTG_BLOCKWISE(norm_l1, XTG_RED_NORM_L1)
XTG_BLOCKWISE(norm_l2, XTG_RED_NORM_L2)
XTG_BLOCKWISE(norm_sq, XTG_RED_NORM_SQ)
XTG_BLOCKWISE(norm_linf, XTG_RED_NORM_LINF)
#undef XTG_BLOCKWISE
#define XTG_BLOCKWISE_P(NAME, CODE)                                                                                \
    template <class E, class BS, class X, std::enable_if_t<!std::is_base_of<reducer_options, X>::value, int> = 0>   \
    inline auto NAME(const E& e, const BS& block_shape, double p, const X& axes, reducer_options o = {}) {          \
        return xblockwise_reducer<CODE, double>(e, block_shape, axes, false, o, p);                                 \
    }                                                                                                               \
    template <class E, class BS>                                                                                    \
    inline auto NAME(const E& e, const BS& block_shape, double p, reducer_options o = {}) {                         \
        return xblockwise_reducer<CODE, double>(e, block_shape, std::vector<std::size_t>{}, true, o, p);            \
    }
XTG_BLOCKWISE_P(norm_lp_to_p, XTG_RED_NORM_LP_TO_P)
XTG_BLOCKWISE_P(norm_lp, XTG_RED_NORM_LP)
#undef XTG_BLOCKWISE_P
}  // namespace blockwise

// ---------------------------------------------------------------------------- index / filter / masked views
// xt::index_view, xt::filter, xt::filtration, xt::masked_view
// (include/xtensor/views/xindex_view.hpp, views/xmasked_view.hpp).  Reading a
// view evaluates it (a gather); writing through it (=, +=, -=, *=, /= with an
// expression or a scalar) writes the selected elements of the underlying
// container or strided view.
namespace detail {
// an lvalue operand is referenced, a temporary expression kept by value
template <class E> using view_closure_t = std::conditional_t<std::is_lvalue_reference<E>::value, E, std::decay_t<E>>;
inline std::shared_ptr<device_buffer> upload_indices(const std::vector<std::vector<std::size_t>>& idx, std::size_t rank) {
    std::vector<int64_t> h;
    h.reserve(idx.size() * rank);
    for (const auto& r : idx) {
        if (r.size() != rank) throw std::out_of_range("index_view: coordinate rank differs from the expression's");
        for (auto v : r) h.push_back((int64_t)v);
    }
    auto b = std::make_shared<device_buffer>(h.size() * sizeof(int64_t));
    if (!h.empty()) check(xtg_memcpy(b->ptr, h.data(), h.size() * sizeof(int64_t), XTG_MEMCPY_H2D, current_stream()));
    return b;
}
template <class V> struct rhs_lowering {
    lowering L;
    std::shared_ptr<void> keep;
    template <class E, std::enable_if_t<is_xexpression<E>::value, int> = 0> explicit rhs_lowering(const E& e) { e.lower(L); }
    template <class S, std::enable_if_t<std::is_arithmetic<S>::value, int> = 0> explicit rhs_lowering(S v) {
        xscalar<V>((V)v).lower(L);
    }
};
template <class E> int32_t rank_of(const E& e) {
    lowering L;
    e.lower(L);
    int32_t r = 0;
    int64_t sh[XTG_MAX_RANK];
    check(xtg_broadcast_shape(&L.e, &r, sh));
    return r;
}
}  // namespace detail

template <class CT> class xindex_view {
public:
    using expression_type = std::decay_t<CT>;
    using value_type = typename expression_type::value_type;
    template <class E> xindex_view(E&& e, std::vector<std::vector<std::size_t>> idx) : m_e(std::forward<E>(e)) {
        m_rank = (std::size_t)detail::rank_of(m_e);
        m_n = idx.size();
        m_idx = detail::upload_indices(idx, m_rank);
    }
    std::vector<std::size_t> shape() const { return {m_n}; }
    std::size_t size() const { return m_n; }
    xarray<value_type> eval() const {
        detail::lowering L;
        m_e.lower(L);
        xarray<value_type> out(std::vector<std::size_t>{m_n});
        xtg_array o = out.xtg_desc();
        detail::resolve_chunked(L);
        detail::check(xtg_gather(&L.e, (const int64_t*)m_idx->ptr, (int64_t)m_n, &o, detail::current_stream()));
        return out;
    }
    operator xarray<value_type>() const { return eval(); }
    value_type operator()(std::size_t i) const { return eval()(i); }
    template <class R> xindex_view& operator=(const R& r) { return apply(r, XTG_SET); }
    template <class R> xindex_view& operator+=(const R& r) { return apply(r, XTG_SET_ADD); }
    template <class R> xindex_view& operator-=(const R& r) { return apply(r, XTG_SET_SUB); }
    template <class R> xindex_view& operator*=(const R& r) { return apply(r, XTG_SET_MUL); }
    template <class R> xindex_view& operator/=(const R& r) { return apply(r, XTG_SET_DIV); }

private:
    template <class R> xindex_view& apply(const R& r, int op) {
        if constexpr (!is_xexpression<R>::value && !std::is_arithmetic<R>::value) {
            auto v = r.eval();  // another view on the right: evaluate it first
            return apply(v, op);
        } else {
            detail::rhs_lowering<value_type> rl(r);
            xtg_array d = m_e.xtg_desc();
            detail::check(
                xtg_scatter(&rl.L.e, (const int64_t*)m_idx->ptr, (int64_t)m_n, op, &d, detail::current_stream()));
            return *this;
        }
    }
    CT m_e;
    std::size_t m_rank = 0, m_n = 0;
    std::shared_ptr<detail::device_buffer> m_idx;
};
template <class E> inline auto index_view(E&& e, std::vector<std::vector<std::size_t>> idx) {
    return xindex_view<detail::view_closure_t<E>>(std::forward<E>(e), std::move(idx));
}

// filter(e, cond): a 1-D view of the elements where cond holds (row-major)
template <class CT, class CC> class xfilter_view {
public:
    using expression_type = std::decay_t<CT>;
    using value_type = typename expression_type::value_type;
    template <class E, class C> xfilter_view(E&& e, C&& c) : m_e(std::forward<E>(e)), m_c(std::forward<C>(c)) {}
    std::size_t size() const {
        detail::lowering C;
        m_c.lower(C);
        int64_t n = 0;
        detail::resolve_chunked(C);
        detail::check(xtg_filter_count(&C.e, &n, detail::current_stream()));
        return (std::size_t)n;
    }
    xarray<value_type> eval() const {
        detail::lowering L, C;
        m_e.lower(L);
        m_c.lower(C);
        xarray<value_type> out(std::vector<std::size_t>{size()});
        xtg_array o = out.xtg_desc();
        detail::resolve_chunked(L);
        detail::resolve_chunked(C);
        detail::check(xtg_filter(&L.e, &C.e, &o, detail::current_stream()));
        return out;
    }
    operator xarray<value_type>() const { return eval(); }
    value_type operator()(std::size_t i) const { return eval()(i); }
    template <class R> xfilter_view& operator=(const R& r) { return apply(r, XTG_SET); }
    template <class R> xfilter_view& operator+=(const R& r) { return apply(r, XTG_SET_ADD); }
    template <class R> xfilter_view& operator-=(const R& r) { return apply(r, XTG_SET_SUB); }
    template <class R> xfilter_view& operator*=(const R& r) { return apply(r, XTG_SET_MUL); }
    template <class R> xfilter_view& operator/=(const R& r) { return apply(r, XTG_SET_DIV); }
    void fill(value_type v) { apply(v, XTG_SET); }

private:
    template <class R> xfilter_view& apply(const R& r, int op) {
        if constexpr (!is_xexpression<R>::value && !std::is_arithmetic<R>::value) {
            auto v = r.eval();  // another view on the right: evaluate it first
            return apply(v, op);
        } else {
            detail::rhs_lowering<value_type> rl(r);
            detail::lowering C;
            m_c.lower(C);
            xtg_array d = m_e.xtg_desc();
            detail::resolve_chunked(rl.L);
            detail::resolve_chunked(C);
            detail::check(xtg_filter_assign(&rl.L.e, &C.e, op, &d, detail::current_stream()));
            return *this;
        }
    }
    CT m_e;
    CC m_c;
};
template <class E, class C> inline auto filter(E&& e, C&& c) {
    return xfilter_view<detail::view_closure_t<E>, detail::view_closure_t<C>>(std::forward<E>(e), std::forward<C>(c));
}
// filtration(e, cond): scalar and computed scalar assignment to the selected elements
template <class E, class C> inline auto filtration(E&& e, C&& c) { return filter(std::forward<E>(e), std::forward<C>(c)); }

template <class CT, class CM> class xmasked_view {
public:
    using expression_type = std::decay_t<CT>;
    using value_type = typename expression_type::value_type;
    template <class E, class M> xmasked_view(E&& e, M&& m) : m_e(std::forward<E>(e)), m_m(std::forward<M>(m)) {}
    template <class R> xmasked_view& operator=(const R& r) { return apply(r, XTG_SET); }
    template <class R> xmasked_view& operator+=(const R& r) { return apply(r, XTG_SET_ADD); }
    template <class R> xmasked_view& operator-=(const R& r) { return apply(r, XTG_SET_SUB); }
    template <class R> xmasked_view& operator*=(const R& r) { return apply(r, XTG_SET_MUL); }
    template <class R> xmasked_view& operator/=(const R& r) { return apply(r, XTG_SET_DIV); }
    void fill(value_type v) { apply(v, XTG_SET); }

private:
    template <class R> xmasked_view& apply(const R& r, int op) {
        static_assert(is_xexpression<R>::value || std::is_arithmetic<R>::value, "masked_view: assign an expression or a scalar");
        detail::rhs_lowering<value_type> rl(r);
        detail::lowering M;
        m_m.lower(M);
        xtg_array d = m_e.xtg_desc();
        detail::resolve_chunked(rl.L);
        detail::resolve_chunked(M);
        detail::check(xtg_masked_assign(&rl.L.e, &M.e, op, &d, detail::current_stream()));
        return *this;
    }
    CT m_e;
    CM m_m;
};
template <class E, class M> inline auto masked_view(E&& e, M&& m) {
    return xmasked_view<detail::view_closure_t<E>, detail::view_closure_t<M>>(std::forward<E>(e), std::forward<M>(m));
}

// ---------------------------------------------------------------------------- .npy files
// xt::load_npy<T, L> / xt::dump_npy (include/xtensor/io/xnpy.hpp:674-800):
// the file streams through libxtg's pinned staging ring straight into the
// device container (a Fortran-order file is reordered on the device; the
// container keeps its row-major strides).
#ifndef XTG_HAVE_LAYOUT_TYPE
#define XTG_HAVE_LAYOUT_TYPE
enum class layout_type { dynamic = 0x00, any = 0xFF, row_major = 0x01, column_major = 0x02 };
#endif

template <class T, layout_type L = layout_type::dynamic> inline xarray<T> load_npy(const std::string& filename) {
    xtg_npy_header h;
    detail::check(xtg_npy_info(filename.c_str(), &h));
    xarray<T> out(std::vector<std::size_t>(h.shape, h.shape + h.rank));
    const xtg_array a = out.xtg_desc();
    detail::check(xtg_npy_load(filename.c_str(), &a, (int32_t)L, detail::current_stream()));
    return out;
}
template <class T, layout_type L = layout_type::dynamic> inline xarray<T> load_npy(std::istream& stream) {
    const std::string buf((std::istreambuf_iterator<char>(stream)), std::istreambuf_iterator<char>());
    xtg_npy_header h;
    detail::check(xtg_npy_info_buffer(buf.data(), buf.size(), &h));
    xarray<T> out(std::vector<std::size_t>(h.shape, h.shape + h.rank));
    const xtg_array a = out.xtg_desc();
    detail::check(xtg_npy_load_buffer(buf.data(), buf.size(), &a, (int32_t)L, detail::current_stream()));
    return out;
}
template <class E> inline void dump_npy(const std::string& filename, const xexpression<E>& e) {
    const auto& ev = xt::eval(e.derived_cast());
    const xtg_array a = ev.xtg_desc();
    detail::check(xtg_npy_save(filename.c_str(), &a, detail::current_stream()));
}
template <class E> inline std::string dump_npy(const xexpression<E>& e) {
    const auto& ev = xt::eval(e.derived_cast());
    const xtg_array a = ev.xtg_desc();
    std::size_t n = 0;
    detail::check(xtg_npy_save_buffer(&a, nullptr, 0, &n, detail::current_stream()));
    std::string out(n, '\0');
    detail::check(xtg_npy_save_buffer(&a, &out[0], n, &n, detail::current_stream()));
    return out;
}

// ---------------------------------------------------------------------------- builders
template <class T, class S> inline xarray<T> ones(const S& s) { return xarray<T>(std::vector<std::size_t>(std::begin(s), std::end(s)), T(1)); }
template <class T, class I> inline xarray<T> ones(std::initializer_list<I> s) { return xarray<T>(std::vector<std::size_t>(s.begin(), s.end()), T(1)); }
template <class T, class S> inline xarray<T> zeros(const S& s) { return xarray<T>(std::vector<std::size_t>(std::begin(s), std::end(s)), T(0)); }
template <class T, class I> inline xarray<T> zeros(std::initializer_list<I> s) { return xarray<T>(std::vector<std::size_t>(s.begin(), s.end()), T(0)); }
template <class T = double> inline xarray<T> arange(std::size_t n) {
    std::vector<T> h(n);
    for (std::size_t i = 0; i < n; ++i) h[i] = (T)i;
    xarray<T> a(std::vector<std::size_t>{n});
    a.upload(h);
    return a;
}

// ---------------------------------------------------------------------------- comparisons / printing
template <class T, std::ptrdiff_t N, class U, std::ptrdiff_t M>
inline bool operator==(const xdevice_container<T, N>& a, const xdevice_container<U, M>& b) {
    if (std::vector<std::size_t>(a.shape().begin(), a.shape().end()) != std::vector<std::size_t>(b.shape().begin(), b.shape().end()))
        return false;
    auto ha = a.to_host();
    auto hb = b.to_host();
    for (std::size_t i = 0; i < ha.size(); ++i)
        if (!(ha[i] == (T)hb[i])) return false;
    return true;
}
template <class T, std::ptrdiff_t N, class U, std::ptrdiff_t M>
inline bool operator!=(const xdevice_container<T, N>& a, const xdevice_container<U, M>& b) { return !(a == b); }

template <class A, class B> inline bool allclose(const A& a, const B& b, double rtol = 1e-5, double atol = 1e-8) {
    auto ea = xt::eval(a);
    auto eb = xt::eval(b);
    auto ha = ea.to_host();
    auto hb = eb.to_host();
    if (ha.size() != hb.size()) return false;
    for (std::size_t i = 0; i < ha.size(); ++i) {
        const double x = (double)ha[i], y = (double)hb[i];
        if (!(std::abs(x - y) <= atol + rtol * std::abs(y)) && !(std::isnan(x) && std::isnan(y))) return false;
    }
    return true;
}

template <class T, std::ptrdiff_t N> inline std::ostream& operator<<(std::ostream& os, const xdevice_container<T, N>& a) {
    auto h = a.to_host();
    os << "{";
    for (std::size_t i = 0; i < h.size(); ++i) os << (i ? ", " : "") << h[i];
    return os << "}";
}

}  // namespace xt

#include "xt_chunked.hpp"
