// xt_chunked.hpp — chunked arrays of the xt:: surface over device chunks
// (xt::xchunked_array / chunked_array, include/xtensor/chunk/xchunked_array.hpp:
// 56-686; xt::xchunked_view / as_chunked, chunk/xchunked_view.hpp; the chunked
// assignment of chunk/xchunked_assign.hpp:185-272), and xt::broadcast of a
// scalar (views/xbroadcast.hpp).  Included by xt.hpp.
//
// Every chunk is a device xarray of chunk_shape (edge chunks keep their
// padding, as in the reference); the chunks of one array share one
// allocation, at a 256-byte aligned distance, so that the library reduces a
// class of equal chunks as one strided array.  Assigning an expression to a chunked array
// evaluates all chunks in one kernel (xtg_chunked_assign); a chunked operand
// of the same grid is read chunk by chunk in place, one of another grid is
// first read into a dense temporary.  Reading a chunked array into a dense
// container is xtg_chunked_to_dense; xt::sum / mean / ... of a chunked array
// reduce through xtg_chunked_reduce (one strided reduction per class of
// equal chunks of the slab).
#pragma once

#include <numeric>

namespace xt {

// ---------------------------------------------------------------------------- broadcast
// xt::broadcast(value, shape): a scalar repeated over `shape`, lowered as a
// one-element device leaf with zero strides.
template <class T> class xbroadcast_scalar : public xexpression<xbroadcast_scalar<T>> {
public:
    using value_type = T;
    template <class S> xbroadcast_scalar(T v, const S& shape) : m_v(v), m_shape(std::begin(shape), std::end(shape)) {}
    const std::vector<std::size_t>& shape() const { return m_shape; }
    std::size_t dimension() const { return m_shape.size(); }
    void lower(detail::lowering& L) const {
        void* p = nullptr;
        detail::check(xtg_malloc(&p, 16, detail::current_stream()));
        std::shared_ptr<void> hold(p, [](void* q) { xtg_free(q, detail::current_stream()); });
        detail::check(xtg_memcpy(p, &m_v, sizeof(T), XTG_MEMCPY_H2D, detail::current_stream()));
        detail::check(xtg_stream_sync(detail::current_stream()));
        L.temps.push_back(hold);
        xtg_array a;
        std::memset(&a, 0, sizeof a);
        a.data = p;
        a.dtype = detail::dtype_of<T>::value;
        a.rank = (int32_t)m_shape.size();
        for (std::size_t i = 0; i < m_shape.size(); ++i) a.shape[i] = (int64_t)m_shape[i];
        const int i = L.leaf(a, this);
        L.node(XTG_OP_LEAF, a.dtype, i);
    }
    bool refers_to(const void*) const { return false; }

private:
    T m_v;
    std::vector<std::size_t> m_shape;
};
template <class T, class S, std::enable_if_t<std::is_arithmetic<T>::value, int> = 0>
inline xbroadcast_scalar<T> broadcast(T v, const S& shape) { return xbroadcast_scalar<T>(v, shape); }
template <class T, class I, std::enable_if_t<std::is_arithmetic<T>::value, int> = 0>
inline xbroadcast_scalar<T> broadcast(T v, std::initializer_list<I> shape) { return xbroadcast_scalar<T>(v, shape); }

// ---------------------------------------------------------------------------- chunked arrays
template <class T> class xchunked_array : public xexpression<xchunked_array<T>> {
public:
    using value_type = T;
    using size_type = std::size_t;
    using shape_type = std::vector<std::size_t>;
    using chunk_type = xarray<T>;
    using chunk_storage_type = std::vector<xarray<T>>;
    using chunk_iterator = typename chunk_storage_type::iterator;
    using const_chunk_iterator = typename chunk_storage_type::const_iterator;

    template <class S1, class S2, std::enable_if_t<!is_xexpression<S1>::value, int> = 0>
    xchunked_array(const S1& shape, const S2& chunk_shape) {
        m_chunk_shape.assign(std::begin(chunk_shape), std::end(chunk_shape));
        reshape_grid(shape_type(std::begin(shape), std::end(shape)));
    }
    // chunked_array(e, chunk_shape): a chunked array with e's shape assigned from e
    template <class E, class S> xchunked_array(const xexpression<E>& e, const S& chunk_shape) {
        m_chunk_shape.assign(std::begin(chunk_shape), std::end(chunk_shape));
        reshape_grid(shape_of(e.derived_cast()));
        noalias_assign(e.derived_cast());
    }
    xchunked_array(const xchunked_array& o) : m_chunk_shape(o.m_chunk_shape) { copy_from(o); }
    xchunked_array(xchunked_array&&) noexcept = default;
    xchunked_array& operator=(const xchunked_array& o) {
        if (this != &o) {
            m_chunk_shape = o.m_chunk_shape;
            copy_from(o);
        }
        return *this;
    }
    xchunked_array& operator=(xchunked_array&&) noexcept = default;

    // a = e: e's shape (xchunked_semantic::operator= rebuilds with this chunk
    // shape when e is larger, xchunked_assign.hpp:222-254)
    template <class E> xchunked_array& operator=(const xexpression<E>& e) {
        resize(shape_of(e.derived_cast()));
        noalias_assign(e.derived_cast());
        return *this;
    }
    template <class E> xchunked_array& operator+=(const E& e) { return *this = *this + e; }
    template <class E> xchunked_array& operator-=(const E& e) { return *this = *this - e; }
    template <class E> xchunked_array& operator*=(const E& e) { return *this = *this * e; }
    template <class E> xchunked_array& operator/=(const E& e) { return *this = *this / e; }

    // geometry
    const shape_type& shape() const noexcept { return m_shape; }
    std::size_t dimension() const noexcept { return m_shape.size(); }
    std::size_t size() const noexcept {
        return std::accumulate(m_shape.begin(), m_shape.end(), std::size_t(1), std::multiplies<std::size_t>());
    }
    const shape_type& chunk_shape() const noexcept { return m_chunk_shape; }
    const shape_type& grid_shape() const noexcept { return m_grid; }
    std::size_t grid_size() const noexcept { return m_chunks.size(); }
    chunk_storage_type& chunks() { return m_chunks; }
    const chunk_storage_type& chunks() const { return m_chunks; }
    chunk_iterator chunk_begin() { return m_chunks.begin(); }
    chunk_iterator chunk_end() { return m_chunks.end(); }
    const_chunk_iterator chunk_begin() const { return m_chunks.begin(); }
    const_chunk_iterator chunk_end() const { return m_chunks.end(); }
    const_chunk_iterator chunk_cbegin() const { return m_chunks.cbegin(); }
    const_chunk_iterator chunk_cend() const { return m_chunks.cend(); }
    template <class S> void resize(const S& s) {
        shape_type ns(std::begin(s), std::end(s));
        if (ns != m_shape) reshape_grid(ns);
    }

    // element access (operator(), element, xchunked_array.hpp:440-470)
    template <class... I> element_ref<T> operator()(I... idx) {
        const std::size_t ix[] = {(std::size_t)idx...};
        return locate(ix, sizeof...(I));
    }
    template <class... I> T operator()(I... idx) const { return const_cast<xchunked_array&>(*this)(idx...); }
    template <class S, std::enable_if_t<!std::is_integral<S>::value, int> = 0> element_ref<T> operator[](const S& idx) {
        std::vector<std::size_t> ix(std::begin(idx), std::end(idx));
        return locate(ix.data(), ix.size());
    }
    template <class It> element_ref<T> element(It first, It last) {
        std::vector<std::size_t> ix(first, last);
        return locate(ix.data(), ix.size());
    }

    // evaluation
    template <class E> void noalias_assign(const E& e) {
        detail::lowering L;
        e.lower(L);
        // a chunked operand of another grid is read into a dense temporary first
        for (int i = 0; i < L.e.n_leaves; ++i) {
            const xtg_chunked* c = L.chunked[(size_t)i];
            if (!c || same_grid(*c)) continue;
            detail::lowering one;
            one.e = L.e;
            one.chunked.assign(L.chunked.size(), nullptr);
            one.chunked[(size_t)i] = c;
            detail::resolve_chunked(one);
            L.e.leaves[i] = one.e.leaves[i];
            L.chunked[(size_t)i] = nullptr;
            L.temps.insert(L.temps.end(), one.temps.begin(), one.temps.end());
        }
        const xtg_chunked d = desc();
        detail::check(xtg_chunked_assign(&L.e, L.chunked.data(), &d, detail::current_stream()));
    }
    xtg_chunked desc() const {
        m_ptrs.clear();
        for (const auto& c : m_chunks) m_ptrs.push_back(const_cast<T*>(c.data()));
        xtg_chunked d;
        std::memset(&d, 0, sizeof d);
        d.chunks = m_ptrs.data();
        d.dtype = detail::dtype_of<T>::value;
        d.rank = (int32_t)m_shape.size();
        for (std::size_t i = 0; i < m_shape.size(); ++i) {
            d.shape[i] = (int64_t)m_shape[i];
            d.chunk_shape[i] = (int64_t)m_chunk_shape[i];
        }
        return d;
    }
    void lower(detail::lowering& L) const {
        m_desc = desc();
        xtg_array a;
        std::memset(&a, 0, sizeof a);
        a.data = m_chunks.empty() ? (void*)this : (void*)m_chunks[0].data();
        a.dtype = detail::dtype_of<T>::value;
        a.rank = (int32_t)m_shape.size();
        int64_t s = 1;
        for (int i = (int)m_shape.size() - 1; i >= 0; --i) {
            a.shape[i] = (int64_t)m_shape[(size_t)i];
            a.strides[i] = s;
            s *= std::max<int64_t>((int64_t)m_shape[(size_t)i], 1);
        }
        const int i = L.chunked_leaf(a, this, &m_desc);
        L.node(XTG_OP_LEAF, a.dtype, i);
    }
    bool refers_to(const void* p) const {
        for (const auto& c : m_chunks)
            if (c.data() == p) return true;
        return false;
    }
    std::vector<T> to_host() const { return xarray<T>(*this).to_host(); }

private:
    template <class E> static shape_type shape_of(const E& e) {
        if constexpr (std::is_same<E, xchunked_array<typename E::value_type>>::value) return e.shape();
        else {
            auto s = detail::broadcast_shape_of(e);
            return shape_type(s.begin(), s.end());
        }
    }
    void reshape_grid(const shape_type& shape) {
        if (shape.size() != m_chunk_shape.size())
            throw std::runtime_error("chunked array: the chunk shape must have the array's rank");
        m_shape = shape;
        m_grid.resize(shape.size());
        std::size_t n = 1;
        for (std::size_t d = 0; d < shape.size(); ++d) {
            if (m_chunk_shape[d] == 0) throw std::runtime_error("chunked array: chunk extents must be positive");
            // chunks per dimension, the edge chunk included (xchunked_array.hpp:601-616)
            m_grid[d] = shape[d] / m_chunk_shape[d] + (shape[d] % m_chunk_shape[d] > 0 ? 1 : 0);
            n *= m_grid[d];
        }
        // one slab, chunks at a 256-byte aligned distance
        std::size_t celems = 1;
        for (auto c : m_chunk_shape) celems *= c;
        const std::size_t dist = (std::max<std::size_t>(celems * sizeof(T), 1) + 255) / 256 * 256;
        auto slab = std::make_shared<detail::device_buffer>(n * dist);
        m_chunks.clear();
        m_chunks.reserve(n);
        for (std::size_t i = 0; i < n; ++i)
            m_chunks.emplace_back(detail::adopt, m_chunk_shape,
                                  std::make_shared<detail::device_buffer>(slab, i * dist, celems * sizeof(T)));
    }
    // a copy with its own slab: every chunk's buffer, padding included
    void copy_from(const xchunked_array& o) {
        reshape_grid(o.m_shape);
        for (std::size_t i = 0; i < m_chunks.size(); ++i)
            detail::check(xtg_memcpy(m_chunks[i].data(), o.m_chunks[i].data(), o.m_chunks[i].size() * sizeof(T),
                                     XTG_MEMCPY_D2D, detail::current_stream()));
    }
    bool same_grid(const xtg_chunked& c) const {
        if (c.rank != (int32_t)m_shape.size()) return false;
        for (std::size_t d = 0; d < m_shape.size(); ++d)
            if (c.shape[d] != (int64_t)m_shape[d] || c.chunk_shape[d] != (int64_t)m_chunk_shape[d]) return false;
        return true;
    }
    // (index of chunk, index in chunk) per dimension (:640-646)
    element_ref<T> locate(const std::size_t* ix, std::size_t n) {
        if (n != m_shape.size()) throw std::runtime_error("chunked array: one index per dimension");
        std::size_t ci = 0, off = 0;
        for (std::size_t d = 0; d < n; ++d) {
            if (ix[d] >= m_shape[d]) throw std::out_of_range("chunked array index out of range");
            const std::size_t of = ix[d] / m_chunk_shape[d];
            ci = ci * m_grid[d] + of;
            off = off * m_chunk_shape[d] + (ix[d] - of * m_chunk_shape[d]);
        }
        return element_ref<T>(m_chunks[ci].data() + off);
    }

    shape_type m_shape, m_chunk_shape, m_grid;
    chunk_storage_type m_chunks;
    mutable std::vector<void*> m_ptrs;
    mutable xtg_chunked m_desc;
};

template <class E> struct is_chunked_t : std::false_type {};
template <class T> struct is_chunked_t<xchunked_array<T>> : std::true_type {};
template <class E> constexpr bool is_chunked(const xexpression<E>&) { return is_chunked_t<E>::value; }
template <class E> constexpr bool is_chunked() { return is_chunked_t<E>::value; }

// chunked_array overloads (xchunked_array.hpp:262-345)
template <class T, class S, std::enable_if_t<!is_xexpression<S>::value, int> = 0>
inline xchunked_array<T> chunked_array(const S& shape, const S& chunk_shape) {
    return xchunked_array<T>(shape, chunk_shape);
}
template <class T, class I>
inline xchunked_array<T> chunked_array(std::initializer_list<I> shape, std::initializer_list<I> chunk_shape) {
    return xchunked_array<T>(std::vector<std::size_t>(shape.begin(), shape.end()),
                             std::vector<std::size_t>(chunk_shape.begin(), chunk_shape.end()));
}
template <class E, class S, std::enable_if_t<!std::is_integral<S>::value, int> = 0>
inline auto chunked_array(const xexpression<E>& e, const S& chunk_shape) {
    return xchunked_array<typename E::value_type>(e, chunk_shape);
}
template <class E, class I> inline auto chunked_array(const xexpression<E>& e, std::initializer_list<I> chunk_shape) {
    return xchunked_array<typename E::value_type>(e, std::vector<std::size_t>(chunk_shape.begin(), chunk_shape.end()));
}
// without a chunk shape: a chunked e's own, any other e's shape (one chunk)
template <class E> inline auto chunked_array(const xexpression<E>& e) {
    const E& d = e.derived_cast();
    if constexpr (is_chunked_t<E>::value) return xchunked_array<typename E::value_type>(e, d.chunk_shape());
    else return xchunked_array<typename E::value_type>(e, detail::broadcast_shape_of(d));
}

// as_chunked(e, chunk_shape) / xchunked_view<E>(e, chunk_shape): assignment
// chunk by chunk into e; the values do not depend on the order the chunks are
// walked in, so it is one assignment of e (chunk/xchunked_view.hpp:77-176).
template <class E> class xchunked_view {
public:
    template <class S> xchunked_view(E& e, const S& chunk_shape) : m_e(e), m_cs(std::begin(chunk_shape), std::end(chunk_shape)) {}
    template <class X> E& operator=(const xexpression<X>& x) {
        noalias(m_e) = x.derived_cast();
        return m_e;
    }
    // the chunks of the view, counted in the grid's row-major order
    struct chunk_iterator {
        std::size_t i;
        chunk_iterator& operator++() { ++i; return *this; }
        chunk_iterator operator++(int) { chunk_iterator t = *this; ++i; return t; }
        bool operator!=(const chunk_iterator& o) const { return i != o.i; }
        bool operator==(const chunk_iterator& o) const { return i == o.i; }
    };
    chunk_iterator chunk_begin() const { return {0}; }
    chunk_iterator chunk_end() const {
        std::size_t n = 1;
        for (std::size_t d = 0; d < m_cs.size(); ++d) n *= m_e.shape()[d] / m_cs[d] + (m_e.shape()[d] % m_cs[d] ? 1 : 0);
        return {n};
    }

private:
    E& m_e;
    std::vector<std::size_t> m_cs;
};
template <class E, class S> inline xchunked_view<E> as_chunked(E& e, const S& chunk_shape) {
    return xchunked_view<E>(e, chunk_shape);
}
template <class E, class I> inline xchunked_view<E> as_chunked(E& e, std::initializer_list<I> chunk_shape) {
    return xchunked_view<E>(e, std::vector<std::size_t>(chunk_shape.begin(), chunk_shape.end()));
}

template <class T, class U, std::ptrdiff_t M> inline bool operator==(const xchunked_array<T>& a, const xdevice_container<U, M>& b) {
    return xarray<T>(a) == b;
}
template <class T, class U, std::ptrdiff_t M> inline bool operator==(const xdevice_container<U, M>& b, const xchunked_array<T>& a) {
    return xarray<T>(a) == b;
}
template <class T, class U> inline bool operator==(const xchunked_array<T>& a, const xchunked_array<U>& b) {
    return xarray<T>(a) == xarray<U>(b);
}

}  // namespace xt
