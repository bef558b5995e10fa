// xtg_chunked.cpp — chunked arrays over device chunks (xt::xchunked_array,
// include/xtensor/chunk/xchunked_array.hpp:56-686; xt::xchunked_view /
// as_chunked, chunk/xchunked_view.hpp; their assignment,
// chunk/xchunked_assign.hpp:185-272).
//
// A chunked array cuts its shape into a grid of ceil(shape / chunk_shape)
// chunks; every chunk is a separate buffer of chunk_shape elements (row-major)
// and the last chunk along a dimension ends inside its buffer (the rest is
// padding), as the reference's resize makes them (xchunked_array.hpp:601-625).
// Element (i0, .., iR-1) lives in chunk (i / chunk_shape) at (i % chunk_shape)
// (get_chunk_indexes_in_dimension, :640-646).
//
// Assignment walks the chunks in the grid's row-major order and assigns the
// matching region of the expression into each (assign_xexpression,
// xchunked_assign.hpp:200-219).  Here that is ONE launch of K12 over
// (chunk, vector inside the chunk's valid region) for the whole grid: per
// chunk a table entry holds the destination chunk's address, each leaf's
// address at the chunk's origin (a dense leaf) or its own chunk (a chunked
// leaf with the same grid), and the chunk's valid extents.  Chunks of equal
// valid extents form a class (at most 2 per dim: full and edge), and the
// table is ordered by class, so the kernel decodes positions inside valid
// regions only and edge chunks cost no idle threads.
// The same kernel copies a chunked array into a dense destination (reading it:
// `noalias(b) = a`, `as_chunked(b, cs) = a`).  Reductions run per chunk
// through the blockwise machinery (xtg_blockwise.cpp).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "xtg_plan.h"
#include "xtg_params.h"

namespace xtgh {

static int kind_of(int64_t s) { return s == 1 ? 0 : (s == 0 ? 1 : 2); }
static bool aligned(const void* p, int64_t bytes) { return ((uintptr_t)p % (uintptr_t)bytes) == 0; }

xtg_status chunk_grid(const xtg_chunked& c, ChunkGrid& g) {
    if (!valid_dtype(c.dtype) || c.rank < 0 || c.rank > XTG_MAX_RANK)
        return fail(XTG_ERR_INVALID, "bad chunked array descriptor");
    g.rank = c.rank;
    g.n = 1;
    for (int d = 0; d < c.rank; ++d) {
        if (c.shape[d] < 0) return fail(XTG_ERR_INVALID, "negative extent");
        if (c.chunk_shape[d] < 1) return fail(XTG_ERR_INVALID, "chunk extents must be positive");
        g.shape[d] = c.shape[d];
        g.cs[d] = c.chunk_shape[d];
        // chunks per dimension, the edge chunk included (xchunked_array.hpp:601-616)
        g.grid[d] = c.shape[d] / c.chunk_shape[d] + (c.shape[d] % c.chunk_shape[d] > 0 ? 1 : 0);
        g.n *= g.grid[d];
    }
    if (g.n > 0 && !c.chunks) return fail(XTG_ERR_INVALID, "null chunk table");
    for (int64_t i = 0; i < g.n; ++i)
        if (!c.chunks[i]) return fail(XTG_ERR_INVALID, "null chunk");
    return XTG_OK;
}

void chunk_coords(const ChunkGrid& g, int64_t i, int64_t* gc) {
    for (int d = g.rank - 1; d >= 0; --d) {
        gc[d] = i % g.grid[d];
        i /= g.grid[d];
    }
}

void chunk_strides(const ChunkGrid& g, int64_t* st) {
    int64_t s = 1;
    for (int d = g.rank - 1; d >= 0; --d) {
        st[d] = s;
        s *= g.cs[d];
    }
}

// Evaluates tree t into every chunk of grid G: destination `dst_c` (chunked,
// grid G) or `dst_d` (dense, G's shape).  leaf_c[slot]: the chunked array of
// that leaf slot (grid G), or null for a dense leaf.
static xtg_status run_chunks(const Tree& t, const std::vector<const xtg_chunked*>& leaf_c, const ChunkGrid& G0,
                             const xtg_chunked* dst_c, const xtg_array* dst_d, int out_dtype, cudaStream_t stream) {
    if (G0.n == 0) return XTG_OK;
    XTG_TRY(ensure_device(nullptr));
    // a 0-d array is one chunk of one element
    ChunkGrid G = G0;
    if (G.rank == 0) {
        G.rank = 1;
        G.shape[0] = G.cs[0] = G.grid[0] = 1;
    }
    const int R = G.rank;
    const int NL = (int)t.leaves.size();
    int64_t cst[XTG_MAX_RANK];
    chunk_strides(G, cst);
    std::vector<std::array<int64_t, XTG_MAX_RANK>> ls(NL);
    for (int l = 0; l < NL; ++l) {
        if (leaf_c[l]) {
            for (int d = 0; d < R; ++d) ls[l][d] = cst[d];
        } else {
            bstrides_to(t.leaves[l], R, G.shape, ls[l].data());
        }
    }
    std::array<int64_t, XTG_MAX_RANK> os{};
    for (int d = 0; d < R; ++d) os[d] = dst_c ? cst[d] : (dst_d->rank ? dst_d->strides[d] : 0);
    const int osz = dt(out_dtype).size;

    // vector width along the innermost dim: whole chunks along it (no edge
    // chunk there), contiguous operands aligned in every chunk
    std::vector<int> kinds(NL);
    int maxsz = osz;
    for (int l = 0; l < NL; ++l) {
        kinds[l] = kind_of(ls[l][R - 1]);
        if (kinds[l] == 0) maxsz = std::max(maxsz, dt(t.leaves[l].dtype).size);
    }
    const int okind = os[R - 1] == 1 ? 0 : 2;
    // valid extent of the edge chunk along the innermost dim
    const int64_t edge_inner = G.shape[R - 1] - (G.grid[R - 1] - 1) * G.cs[R - 1];
    auto vec_ok = [&](int v) {
        if (v == 1) return true;
        if (G.cs[R - 1] % v || edge_inner % v) return false;
        auto strides_ok = [&](const std::array<int64_t, XTG_MAX_RANK>& st) {
            for (int d = 0; d + 1 < R; ++d)
                if (st[d] % v) return false;
            return true;
        };
        if (okind == 0) {
            if (!strides_ok(os)) return false;
            if (dst_c) {
                for (int64_t i = 0; i < G.n; ++i)
                    if (!aligned(dst_c->chunks[i], (int64_t)v * osz)) return false;
            } else if (!aligned(dst_d->data, (int64_t)v * osz)) {
                return false;
            }
        }
        for (int l = 0; l < NL; ++l) {
            if (kinds[l] != 0) continue;
            const int sz = dt(t.leaves[l].dtype).size;
            if (!strides_ok(ls[l])) return false;
            if (leaf_c[l]) {
                for (int64_t i = 0; i < G.n; ++i)
                    if (!aligned(leaf_c[l]->chunks[i], (int64_t)v * sz)) return false;
            } else if (!aligned(t.leaves[l].data, (int64_t)v * sz)) {
                return false;
            }
        }
        return true;
    };
    int vec = 16 / maxsz;
    if (vec < 1) vec = 1;
    while (vec > 1 && !vec_ok(vec)) vec >>= 1;

    // classes of equal valid extents: per dim, full chunks and (when the
    // shape does not divide) the edge chunk; class id = mixed-radix digits
    int nkind[XTG_MAX_RANK];
    int n_cls = 1;
    for (int d = 0; d < R; ++d) {
        nkind[d] = (G.grid[d] > 1 && G.shape[d] % G.cs[d]) ? 2 : 1;
        n_cls *= nkind[d];
    }
    const bool pad = n_cls > XTG_KCHUNK_CLS;
    auto class_of = [&](const int64_t* gc) {
        int c = 0;
        for (int d = 0; d < R; ++d) c = c * nkind[d] + (nkind[d] == 2 && gc[d] == G.grid[d] - 1 ? 1 : 0);
        return pad ? 0 : c;
    };
    if (pad) n_cls = 1;
    std::vector<int64_t> cls_count((size_t)n_cls, 0), cls_first((size_t)n_cls, 0);
    std::vector<std::array<int64_t, XTG_MAX_RANK>> cls_ext((size_t)n_cls);
    std::vector<int> cls_of((size_t)G.n);
    for (int64_t i = 0; i < G.n; ++i) {
        int64_t gc[XTG_MAX_RANK];
        chunk_coords(G, i, gc);
        const int c = class_of(gc);
        cls_of[(size_t)i] = c;
        if (cls_count[(size_t)c]++ == 0)
            for (int d = 0; d < R; ++d)
                cls_ext[(size_t)c][d] = pad ? G.cs[d] : std::min(G.cs[d], G.shape[d] - gc[d] * G.cs[d]);
    }
    for (int c = 1; c < n_cls; ++c) cls_first[(size_t)c] = cls_first[(size_t)c - 1] + cls_count[(size_t)c - 1];

    // the chunk table, class by class (grid row-major inside a class)
    std::vector<xtg::ChunkEntry> tab((size_t)G.n);
    std::vector<int64_t> fill(cls_first);
    for (int64_t i = 0; i < G.n; ++i) {
        xtg::ChunkEntry& e = tab[(size_t)fill[(size_t)cls_of[(size_t)i]]++];
        memset(&e, 0, sizeof e);
        int64_t gc[XTG_MAX_RANK];
        chunk_coords(G, i, gc);
        for (int d = 0; d < R; ++d) e.ext[d] = std::min(G.cs[d], G.shape[d] - gc[d] * G.cs[d]);
        for (int l = 0; l < NL; ++l) {
            if (leaf_c[l]) {
                e.leaf[l] = leaf_c[l]->chunks[i];
            } else {
                int64_t o = 0;
                for (int d = 0; d < R; ++d) o += gc[d] * G.cs[d] * ls[l][d];
                e.leaf[l] = (const char*)t.leaves[l].data + o * dt(t.leaves[l].dtype).size;
            }
        }
        if (dst_c) {
            e.out = dst_c->chunks[i];
        } else {
            int64_t o = 0;
            for (int d = 0; d < R; ++d) o += gc[d] * G.cs[d] * os[d];
            e.out = (char*)dst_d->data + o * osz;
        }
    }
    void* dtab = nullptr;
    const size_t tab_bytes = tab.size() * sizeof(xtg::ChunkEntry);
    XTG_TRY(scratch_alloc(&dtab, tab_bytes, stream));
    if (recorder()) recorder()->nocache = true;
    if (!dry_run()) {
        const cudaError_t ce = cudaMemcpyAsync(dtab, tab.data(), tab_bytes, cudaMemcpyHostToDevice, stream);
        if (ce != cudaSuccess) {
            scratch_free(dtab, stream);
            return cuda_fail(ce, "chunk table upload");
        }
    }

    xtg::ChunkParams p;
    memset(&p, 0, sizeof p);
    p.n_cls = n_cls;
    int64_t total = 0, largest = 0;
    for (int c = 0; c < n_cls; ++c) {
        xtg::ChunkClass& K = p.cls[c];
        int64_t nvec = 1;
        for (int d = 0; d < R; ++d) {
            K.sp.shape[d] = d == R - 1 ? cls_ext[(size_t)c][d] / vec : cls_ext[(size_t)c][d];
            nvec *= K.sp.shape[d];
        }
        K.sp.nvec = nvec;
        K.first = cls_first[(size_t)c];
        K.count = cls_count[(size_t)c];
        total += nvec * K.count;
        largest = std::max<int64_t>(largest, nvec * K.count);
    }
    const bool big = largest > (int64_t)0xFFFFFFF0ll;
    if (!big)
        for (int c = 0; c < n_cls; ++c) {
            xtg::ChunkClass& K = p.cls[c];
            for (int d = 0; d < R; ++d) K.sp.fd[d] = make_fd((uint64_t)K.sp.shape[d]);
            K.fdn = make_fd((uint64_t)K.sp.nvec);
        }
    p.tab = (const xtg::ChunkEntry*)dtab;
    for (int l = 0; l < NL; ++l)
        for (int d = 0; d < R; ++d) p.leaf_strides[l][d] = ls[l][d];
    for (int d = 0; d < R; ++d) p.out_strides[d] = os[d];
    for (size_t i = 0; i < t.scalars.size(); ++i) p.scal.v[i] = t.scalars[i];

    std::vector<int> map(NL);
    for (int l = 0; l < NL; ++l) map[l] = l;
    std::string ls_s = "xtg::LeafSet<";
    for (int l = 0; l < NL; ++l) {
        if (l) ls_s += ", ";
        ls_s += std::string("xtg::LeafSpec<") + dt(t.leaves[l].dtype).cname + ", " + std::to_string(kinds[l]) + ">";
    }
    ls_s += ">";
    const int U = vec * maxsz >= 16 ? 4 : 8;
    const std::string name = "xtg::k_assign_chunks<" + tree_type(t, t.root, map) + ", " + ls_s + ", " +
                             dt(out_dtype).cname + ", " + std::to_string(okind) + ", " + std::to_string(vec) + ", " +
                             std::to_string(R) + ", " + std::to_string(U) + ", " + (big ? "true" : "false") + ", " +
                             (pad ? "true" : "false") + ">";
    Kernel* k;
    xtg_status st = get_kernel(name, 256, &k);
    if (st == XTG_OK) {
        DeviceInfo* dev;
        ensure_device(&dev);
        const int64_t need = (total + 256 * U - 1) / (256 * U);
        const int64_t cap = (int64_t)k->max_blocks_per_sm * dev->sm_count;
        st = launch(k, (unsigned)std::max<int64_t>(1, std::min(need, cap)), 256, &p, stream);
    }
    const xtg_status fs = scratch_free(dtab, stream);
    return st != XTG_OK ? st : fs;
}

// Tree of `e` with chunked leaf i described by chunked_leaves[i]: its entry in
// the expression gives dtype and shape; its address is replaced by the first
// chunk's (a stand-in unique to the array, so that leaf de-duplication keeps
// different chunked arrays apart).
static xtg_status chunked_tree(const xtg_expr* e, const xtg_chunked* const* chunked_leaves, bool demote, Tree& t,
                               std::vector<const xtg_chunked*>& leaf_c) {
    xtg_expr ex = *e;
    std::vector<const xtg_chunked*> by_expr((size_t)std::max(0, ex.n_leaves), nullptr);
    for (int i = 0; chunked_leaves && i < ex.n_leaves; ++i) {
        const xtg_chunked* c = chunked_leaves[i];
        if (!c) continue;
        ChunkGrid g;
        XTG_TRY(chunk_grid(*c, g));
        xtg_array& a = ex.leaves[i];
        a.dtype = c->dtype;
        a.rank = c->rank;
        int64_t s = 1;
        for (int d = c->rank - 1; d >= 0; --d) {
            a.shape[d] = c->shape[d];
            a.strides[d] = s;
            s *= std::max<int64_t>(c->shape[d], 1);
        }
        a.data = g.n ? c->chunks[0] : (void*)c;
        by_expr[(size_t)i] = c;
    }
    XTG_TRY(build_tree(&ex, demote, t));
    leaf_c.assign(t.leaves.size(), nullptr);
    for (int i = 0; i < ex.n_leaves; ++i) {
        const int slot = i < (int)t.expr_slot.size() ? t.expr_slot[(size_t)i] : -1;
        if (slot >= 0 && by_expr[(size_t)i]) leaf_c[(size_t)slot] = by_expr[(size_t)i];
    }
    return XTG_OK;
}

static bool same_grid(const xtg_chunked& a, const ChunkGrid& g) {
    if (a.rank != g.rank) return false;
    for (int d = 0; d < g.rank; ++d)
        if (a.shape[d] != g.shape[d] || a.chunk_shape[d] != g.cs[d]) return false;
    return true;
}

}  // namespace xtgh

using namespace xtgh;

extern "C" {

xtg_status xtg_chunked_assign(const xtg_expr* e, const xtg_chunked* const* chunked_leaves, const xtg_chunked* dst,
                              xtg_stream stream) {
    begin_call();
    if (!e || !dst) return fail(XTG_ERR_INVALID, "null argument");
    ChunkGrid G;
    XTG_TRY(chunk_grid(*dst, G));
    Tree t;
    std::vector<const xtg_chunked*> leaf_c;
    XTG_TRY(chunked_tree(e, chunked_leaves, opt("fp32_compute", 1) != 0 && dst->dtype != XTG_FLOAT64, t, leaf_c));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics in a chunked assignment");
    // the expression broadcasts to the destination's shape
    if (t.rank > G.rank) return fail(XTG_ERR_SHAPE, "destination rank is smaller than the expression's");
    for (int i = 0; i < t.rank; ++i) {
        const int d = G.rank - t.rank + i;
        if (t.shape[i] != G.shape[d] && t.shape[i] != 1)
            return fail(XTG_ERR_SHAPE, "destination shape does not match the expression shape");
    }
    for (size_t l = 0; l < leaf_c.size(); ++l) {
        if (leaf_c[l] && !same_grid(*leaf_c[l], G))
            return fail(XTG_ERR_UNSUPPORTED, "a chunked operand with another chunk grid than the destination's");
        if (!leaf_c[l] && !t.leaves[l].data) return fail(XTG_ERR_INVALID, "null leaf data");
    }
    return run_chunks(t, leaf_c, G, dst, nullptr, dst->dtype, (cudaStream_t)stream);
}

xtg_status xtg_chunked_to_dense(const xtg_chunked* src, const xtg_array* dst, xtg_stream stream) {
    begin_call();
    if (!src || !dst) return fail(XTG_ERR_INVALID, "null argument");
    ChunkGrid G;
    XTG_TRY(chunk_grid(*src, G));
    if (dst->rank != src->rank) return fail(XTG_ERR_SHAPE, "destination rank differs from the chunked array's");
    for (int d = 0; d < dst->rank; ++d)
        if (dst->shape[d] != src->shape[d]) return fail(XTG_ERR_SHAPE, "destination shape mismatch");
    if (G.n && !dst->data) return fail(XTG_ERR_INVALID, "null destination data");
    xtg_expr e;
    memset(&e, 0, sizeof e);
    e.n_nodes = 1;
    e.nodes[0].op = XTG_OP_LEAF;
    e.nodes[0].dtype = src->dtype;
    e.n_leaves = 1;
    const xtg_chunked* one[1] = {src};
    Tree t;
    std::vector<const xtg_chunked*> leaf_c;
    XTG_TRY(chunked_tree(&e, one, false, t, leaf_c));
    return run_chunks(t, leaf_c, G, nullptr, dst, dst->dtype, (cudaStream_t)stream);
}

}  // extern "C"
