// xtg_views.cpp — reading and assigning through xt::index_view, xt::filter,
// xt::filtration and xt::masked_view
// (include/xtensor/views/xindex_view.hpp:54-206, 786-850;
//  include/xtensor/views/xmasked_view.hpp:63-240).
//
//  * masked_view(dst, mask) op= src lowers to the elementwise tree
//    where(mask, dst op src, dst) assigned in place (the destination is read
//    and written at the same positions);
//  * index_view reads are a gather and writes a scatter over a device list of
//    coordinates (K10 k_indexed, coordinates checked on the device);
//  * filter(e, cond) and filtration(dst, cond) run by tiles of 4096
//    row-major positions: per-tile counts of cond, their inclusive scan, then
//    each tile's selected elements go to the tile's offset plus their rank
//    in the tile — the order of argwhere (xindex_view.hpp:821-826).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "xtg_plan.h"

namespace xtgh {

namespace {

xtg_status append_expr(xtg_expr& d, const xtg_expr* s) {
    if (!s) return fail(XTG_ERR_INVALID, "null expression");
    if (s->n_nodes <= 0 || s->n_nodes > XTG_MAX_NODES || s->n_leaves < 0 || s->n_leaves > XTG_MAX_LEAVES)
        return fail(XTG_ERR_INVALID, "bad expression");
    if (d.n_nodes + s->n_nodes > XTG_MAX_NODES || d.n_leaves + s->n_leaves > XTG_MAX_LEAVES)
        return fail(XTG_ERR_UNSUPPORTED, "composed view expression is too large");
    const int base = d.n_leaves;
    for (int l = 0; l < s->n_leaves; ++l) d.leaves[base + l] = s->leaves[l];
    d.n_leaves += s->n_leaves;
    for (int i = 0; i < s->n_nodes; ++i) {
        xtg_node x = s->nodes[i];
        if (x.op == XTG_OP_LEAF) x.arg += base;
        d.nodes[d.n_nodes++] = x;
    }
    return XTG_OK;
}
xtg_status push_leaf(xtg_expr& d, const xtg_array& a) {
    if (d.n_nodes >= XTG_MAX_NODES || d.n_leaves >= XTG_MAX_LEAVES)
        return fail(XTG_ERR_UNSUPPORTED, "composed view expression is too large");
    d.leaves[d.n_leaves] = a;
    xtg_node x;
    memset(&x, 0, sizeof x);
    x.op = XTG_OP_LEAF;
    x.dtype = a.dtype;
    x.arg = d.n_leaves++;
    d.nodes[d.n_nodes++] = x;
    return XTG_OK;
}
xtg_status push_op(xtg_expr& d, int op, int arg = 0) {
    if (d.n_nodes >= XTG_MAX_NODES) return fail(XTG_ERR_UNSUPPORTED, "composed view expression is too large");
    xtg_node x;
    memset(&x, 0, sizeof x);
    x.op = op;
    x.dtype = -1;
    x.arg = arg;
    d.nodes[d.n_nodes++] = x;
    return XTG_OK;
}
int set_opcode(int op) {
    switch (op) {
        case XTG_SET_ADD: return XTG_OP_ADD;
        case XTG_SET_SUB: return XTG_OP_SUB;
        case XTG_SET_MUL: return XTG_OP_MUL;
        case XTG_SET_DIV: return XTG_OP_DIV;
        default: return -1;
    }
}

std::string leafset_of(const Tree& t) {
    std::string s = "xtg::LeafSet<";
    for (size_t i = 0; i < t.leaves.size(); ++i) {
        if (i) s += ", ";
        s += std::string("xtg::LeafSpec<") + dt(t.leaves[i].dtype).cname + ", 2>";
    }
    return s + ">";
}

unsigned grid_n(Kernel* k, int64_t n) {
    DeviceInfo* dev;
    ensure_device(&dev);
    const int64_t cap = (int64_t)k->max_blocks_per_sm * dev->sm_count;
    return (unsigned)std::max<int64_t>(1, std::min((n + 255) / 256, cap));
}

bool same_shape(const Tree& t, const xtg_array& a) {
    if (t.rank != a.rank) return false;
    for (int d = 0; d < a.rank; ++d)
        if (t.shape[d] != a.shape[d]) return false;
    return true;
}

// Filters run by tiles of 4096 row-major positions: per-tile counts of the
// condition (K11 k_filter_count), their inclusive scan (the accumulator
// kernels, int64), then the compaction / write kernel.  FilterRun holds the
// scratch (counts + scan) and the condition's part of the parameters.
struct FilterRun {
    xtg::FilterParams p;
    Tree tc;
    void* scratch = nullptr;
    int64_t ntiles = 0;
    bool big = false;
    bool v16 = false;  // one flat dim, condition leaves contiguous (aligned) or broadcast: 16-byte loads
    int rank = 1;  // of the position space after merging dims that are contiguous for every array
    std::string ctree, cls;
    std::vector<std::array<int64_t, XTG_MAX_RANK>> extra;  // the callers' position strides, merged alike
};

// `extra`: strides over the filtered shape of the other arrays the tile pass
// addresses by position (the value leaves of a read, the destination of an
// assignment).  Dims that are contiguous for the condition and all of them
// merge (row-major order is kept), so a contiguous filter walks one flat dim.
xtg_status filter_prepare(const xtg_expr* cond, int rank, const int64_t* shape, FilterRun& F, cudaStream_t stream,
                          const std::vector<std::array<int64_t, XTG_MAX_RANK>>& extra = {}) {
    XTG_TRY(build_tree(cond, false, F.tc));
    if (F.tc.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside a filter condition");
    if (F.tc.rank != rank) return fail(XTG_ERR_SHAPE, "condition shape differs from the filtered expression's");
    for (int d = 0; d < rank; ++d)
        if (F.tc.shape[d] != shape[d]) return fail(XTG_ERR_SHAPE, "condition shape differs from the filtered expression's");
    memset(&F.p, 0, sizeof F.p);
    int64_t n = 1;
    for (int d = 0; d < rank; ++d) n *= shape[d];
    F.p.n = n;
    F.big = n > 0xFFFFFFF0ll;
    const int NL = (int)F.tc.leaves.size();
    Dims D;
    D.R = rank;
    for (int d = 0; d < rank; ++d) D.shape[d] = shape[d];
    D.st.resize(NL + extra.size());
    for (int l = 0; l < NL; ++l) {
        F.p.cleaf[l] = F.tc.leaves[l].data;
        D.st[l].fill(0);
        bstrides_to(F.tc.leaves[l], rank, shape, D.st[l].data());
    }
    for (size_t e = 0; e < extra.size(); ++e) D.st[NL + e] = extra[e];
    if (D.st.empty()) D.st.resize(1);
    collapse(D);
    if (D.R == 0) {  // every extent 1: one position
        D.R = 1;
        D.shape[0] = 1;
        for (auto& st : D.st) st[0] = 0;
    }
    F.rank = D.R;
    for (int d = 0; d < D.R; ++d) {
        F.p.shape[d] = D.shape[d];
        F.p.fd[d] = make_fd((uint64_t)std::max<int64_t>(D.shape[d], 1));
    }
    for (int l = 0; l < NL; ++l)
        for (int d = 0; d < D.R; ++d) F.p.cls[l][d] = D.st[l][d];
    F.extra.assign(D.st.begin() + NL, D.st.begin() + NL + extra.size());
    F.v16 = F.rank == 1;
    for (int l = 0; F.v16 && l < NL; ++l) {
        const int64_t st = F.p.cls[l][0];
        F.v16 = st == 0 || (st == 1 && ((uintptr_t)F.tc.leaves[l].data % 16) == 0);
    }
    for (size_t i = 0; i < F.tc.scalars.size(); ++i) F.p.cscal.v[i] = F.tc.scalars[i];
    std::vector<int> map(NL);
    for (int l = 0; l < NL; ++l) map[l] = l;
    F.ctree = tree_type(F.tc, F.tc.root, map);
    F.cls = leafset_of(F.tc);
    F.ntiles = (n + 4095) / 4096;
    if (F.ntiles == 0) return XTG_OK;
    // scratch: int32 counts, then int64 inclusive counts
    const size_t cbytes = (size_t)((F.ntiles * 4 + 15) / 16 * 16);
    XTG_TRY(scratch_alloc(&F.scratch, cbytes + (size_t)F.ntiles * 8, stream));
    F.p.tcount = (int*)F.scratch;
    F.p.tincl = (const long long*)((char*)F.scratch + cbytes);
    if (recorder()) recorder()->nocache = true;  // scratch addresses are baked into several parameter blocks
    Kernel* k;
    XTG_TRY(get_kernel("xtg::k_filter_count<" + F.ctree + ", " + F.cls + ", " + std::to_string(F.rank) + ", " +
                           (F.big ? "true" : "false") + ", " + (F.v16 ? "true" : "false") + ">",
                       256, &k));
    XTG_TRY(launch(k, grid_n(k, F.ntiles * 256), 256, &F.p, stream));
    // inclusive scan of the int32 counts into int64
    xtg_expr ce;
    memset(&ce, 0, sizeof ce);
    xtg_array ca;
    memset(&ca, 0, sizeof ca);
    ca.data = F.scratch;
    ca.dtype = XTG_INT32;
    ca.rank = 1;
    ca.shape[0] = F.ntiles;
    ca.strides[0] = 1;
    XTG_TRY(push_leaf(ce, ca));
    xtg_array ia = ca;
    ia.data = (void*)F.p.tincl;
    ia.dtype = XTG_INT64;
    return accumulate_call(&ce, XTG_ACC_CUMSUM, 0, 0, XTG_INT64, &ia, stream);
}

xtg_status filter_total(const FilterRun& F, int64_t* count, cudaStream_t stream) {
    if (F.ntiles == 0 || dry_run()) {
        *count = 0;
        return XTG_OK;
    }
    long long c = 0;
    XTG_CUDA(cudaMemcpyAsync(&c, F.p.tincl + (F.ntiles - 1), 8, cudaMemcpyDeviceToHost, stream));
    XTG_CUDA(cudaStreamSynchronize(stream));
    *count = c;
    return XTG_OK;
}

// The strides the tile pass addresses by position, before merging: the
// value leaves of a read (mode 0) or the destination of an assignment.
std::vector<std::array<int64_t, XTG_MAX_RANK>> filter_extra(const Tree& tv, int mode, int rank, const int64_t* shape,
                                                            const xtg_array& dst) {
    std::vector<std::array<int64_t, XTG_MAX_RANK>> ex;
    if (mode == 0) {
        for (const auto& L : tv.leaves) {
            ex.emplace_back();
            ex.back().fill(0);
            bstrides_to(L, rank, shape, ex.back().data());
        }
    } else {
        ex.emplace_back();
        ex.back().fill(0);
        for (int d = 0; d < dst.rank; ++d) ex.back()[d] = dst.shape[d] == 1 ? 0 : dst.strides[d];
    }
    return ex;
}

xtg_status filter_launch(FilterRun& F, const Tree& tv, int mode, int op, const xtg_array& dst, cudaStream_t stream) {
    const int NL = (int)tv.leaves.size();
    for (int l = 0; l < NL; ++l) {
        F.p.vleaf[l] = tv.leaves[l].data;
        if (mode == 0) {
            for (int d = 0; d < F.rank; ++d) F.p.vls[l][d] = F.extra[l][d];
        } else {
            int64_t one = std::max<int64_t>(1, tv.rank ? tv.shape[0] : 1);
            bstrides_to(tv.leaves[l], 1, &one, reinterpret_cast<int64_t*>(F.p.vls[l]));
        }
    }
    for (size_t i = 0; i < tv.scalars.size(); ++i) F.p.vscal.v[i] = tv.scalars[i];
    F.p.dst = dst.data;
    if (mode == 0) {
        F.p.ds[0] = dst.strides[0];  // the 1-D compacted result
    } else {
        for (int d = 0; d < F.rank; ++d) F.p.ds[d] = F.extra[0][d];
    }
    const int rank = F.rank;
    std::vector<int> map(NL);
    for (int l = 0; l < NL; ++l) map[l] = l;
    const int vt = tv.nodes[tv.root].dtype;
    const int ct = promote(dst.dtype, vt);
    std::string name = "xtg::k_filter_tile<" + F.ctree + ", " + F.cls + ", " + tree_type(tv, tv.root, map) + ", " +
                       leafset_of(tv) + ", " + dt(vt).cname + ", " + dt(dst.dtype).cname + ", " + dt(ct).cname + ", " +
                       std::to_string(mode) + ", " + std::to_string(rank) + ", " + std::to_string(op) + ", " +
                       (F.big ? "true" : "false") + ", " + (F.v16 ? "true" : "false") + ">";
    Kernel* k;
    XTG_TRY(get_kernel(name, 256, &k));
    return launch(k, grid_n(k, F.ntiles * 256), 256, &F.p, stream);
}

// K10 launch
xtg_status launch_indexed(const Tree& t, int mode, int op, int rank, const int64_t* shape, const long long* idx,
                          int64_t n, const xtg_array& dst, cudaStream_t stream) {
    const int NL = (int)t.leaves.size();
    xtg::IndexParams p;
    memset(&p, 0, sizeof p);
    p.n = n;
    p.rank = rank;
    for (int d = 0; d < rank; ++d) {
        p.shape[d] = shape[d];
        p.fd[d] = make_fd((uint64_t)std::max<int64_t>(shape[d], 1));
    }
    p.idx = idx;
    for (int l = 0; l < NL; ++l) {
        p.leaf[l] = t.leaves[l].data;
        if (mode == 0) {
            bstrides_to(t.leaves[l], rank, shape, reinterpret_cast<int64_t*>(p.ls[l]));
        } else {
            int64_t one = n;  // the value tree runs over a 1-D space of n (or count) elements
            bstrides_to(t.leaves[l], 1, &one, reinterpret_cast<int64_t*>(p.ls[l]));
        }
    }
    p.dst = dst.data;
    for (int d = 0; d < dst.rank; ++d) p.ds[d] = dst.strides[d];
    for (size_t i = 0; i < t.scalars.size(); ++i) p.scal.v[i] = t.scalars[i];
    XTG_TRY(device_error_word(&p.err));
    std::vector<int> map(NL);
    for (int l = 0; l < NL; ++l) map[l] = l;
    const int vt = t.nodes[t.root].dtype;
    const int ct = promote(dst.dtype, vt);
    std::string name = "xtg::k_indexed<" + tree_type(t, t.root, map) + ", " + leafset_of(t) + ", " + dt(vt).cname +
                       ", " + dt(dst.dtype).cname + ", " + dt(ct).cname + ", " + std::to_string(mode) + ", " +
                       std::to_string(rank) + ", " + std::to_string(op) + ">";
    Kernel* k;
    XTG_TRY(get_kernel(name, 256, &k));
    return launch(k, grid_n(k, n), 256, &p, stream);
}

xtg_status check_set_op(int op) {
    if (op < XTG_SET || op > XTG_SET_DIV) return fail(XTG_ERR_INVALID, "bad assignment operator");
    return XTG_OK;
}

}  // namespace

}  // namespace xtgh

using namespace xtgh;

extern "C" {

xtg_status xtg_masked_assign(const xtg_expr* src, const xtg_expr* mask, int32_t op, const xtg_array* dst,
                             xtg_stream stream) {
    begin_call();
    if (!dst || !src || !mask) return fail(XTG_ERR_INVALID, "null argument");
    XTG_TRY(check_set_op(op));
    xtg_expr e;
    memset(&e, 0, sizeof e);
    XTG_TRY(append_expr(e, mask));
    if (op == XTG_SET) {
        XTG_TRY(append_expr(e, src));
    } else {
        XTG_TRY(push_leaf(e, *dst));
        XTG_TRY(append_expr(e, src));
        XTG_TRY(push_op(e, set_opcode(op)));
    }
    XTG_TRY(push_leaf(e, *dst));
    XTG_TRY(push_op(e, XTG_OP_WHERE));
    Tree t;
    XTG_TRY(build_tree(&e, opt("fp32_compute", 1) != 0 && dst->dtype != XTG_FLOAT64, t));
    return assign_guarded(t, dst, (cudaStream_t)stream);
}

xtg_status xtg_gather(const xtg_expr* e, const int64_t* indices, int64_t n, const xtg_array* out, xtg_stream stream) {
    begin_call();
    if (!out || (n > 0 && !indices)) return fail(XTG_ERR_INVALID, "null argument");
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0 && out->dtype != XTG_FLOAT64, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside an index view");
    if (t.rank < 1) return fail(XTG_ERR_INVALID, "index view of a 0-d expression");
    if (out->rank != 1 || out->shape[0] != n) return fail(XTG_ERR_SHAPE, "index view result must be 1-D of n elements");
    if (n == 0) return XTG_OK;
    return launch_indexed(t, 0, 0, t.rank, t.shape, (const long long*)indices, n, *out, (cudaStream_t)stream);
}

xtg_status xtg_scatter(const xtg_expr* src, const int64_t* indices, int64_t n, int32_t op, const xtg_array* dst,
                       xtg_stream stream) {
    begin_call();
    if (!dst || (n > 0 && !indices)) return fail(XTG_ERR_INVALID, "null argument");
    XTG_TRY(check_set_op(op));
    Tree t;
    XTG_TRY(build_tree(src, opt("fp32_compute", 1) != 0 && dst->dtype != XTG_FLOAT64, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside an index view");
    if (t.rank > 1 || (t.rank == 1 && t.shape[0] != n && t.shape[0] != 1))
        return fail(XTG_ERR_BROADCAST, "assigned values do not broadcast to the index view's length");
    if (dst->rank < 1) return fail(XTG_ERR_INVALID, "index view of a 0-d array");
    if (n == 0) return XTG_OK;
    return launch_indexed(t, 1, op, dst->rank, dst->shape, (const long long*)indices, n, *dst, (cudaStream_t)stream);
}

xtg_status xtg_filter_count(const xtg_expr* cond, int64_t* count, xtg_stream stream) {
    begin_call();
    if (!count) return fail(XTG_ERR_INVALID, "null argument");
    Tree tc;
    XTG_TRY(build_tree(cond, false, tc));
    FilterRun F;
    xtg_status st = filter_prepare(cond, tc.rank, tc.shape, F, (cudaStream_t)stream);
    if (st == XTG_OK) st = filter_total(F, count, (cudaStream_t)stream);
    xtg_status fs = F.scratch ? scratch_free(F.scratch, (cudaStream_t)stream) : XTG_OK;
    return st != XTG_OK ? st : fs;
}

xtg_status xtg_filter(const xtg_expr* e, const xtg_expr* cond, const xtg_array* out, xtg_stream stream) {
    begin_call();
    if (!out) return fail(XTG_ERR_INVALID, "null destination");
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0 && out->dtype != XTG_FLOAT64, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside a filter");
    if (t.rank < 1) return fail(XTG_ERR_INVALID, "filter of a 0-d expression");
    if (out->rank != 1) return fail(XTG_ERR_SHAPE, "filter result must be 1-D");
    FilterRun F;
    xtg_status st = filter_prepare(cond, t.rank, t.shape, F, (cudaStream_t)stream, filter_extra(t, 0, t.rank, t.shape, *out));
    int64_t count = 0;
    if (st == XTG_OK) st = filter_total(F, &count, (cudaStream_t)stream);
    if (st == XTG_OK && !dry_run() && out->shape[0] != count)
        st = fail(XTG_ERR_SHAPE, "filter result must be 1-D of xtg_filter_count elements");
    if (st == XTG_OK && F.ntiles) st = filter_launch(F, t, 0, 0, *out, (cudaStream_t)stream);
    xtg_status fs = F.scratch ? scratch_free(F.scratch, (cudaStream_t)stream) : XTG_OK;
    return st != XTG_OK ? st : fs;
}

xtg_status xtg_filter_assign(const xtg_expr* src, const xtg_expr* cond, int32_t op, const xtg_array* dst,
                             xtg_stream stream) {
    begin_call();
    if (!dst) return fail(XTG_ERR_INVALID, "null destination");
    XTG_TRY(check_set_op(op));
    Tree t;
    XTG_TRY(build_tree(src, opt("fp32_compute", 1) != 0 && dst->dtype != XTG_FLOAT64, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside a filter");
    if (t.rank > 1) return fail(XTG_ERR_BROADCAST, "values assigned through a filter must be 1-D or a scalar");
    if (dst->rank < 1) return fail(XTG_ERR_INVALID, "filter of a 0-d array");
    FilterRun F;
    xtg_status st = filter_prepare(cond, dst->rank, dst->shape, F, (cudaStream_t)stream,
                                   filter_extra(t, 1, dst->rank, dst->shape, *dst));
    if (st == XTG_OK && t.rank == 1 && t.shape[0] != 1) {
        int64_t count = 0;
        st = filter_total(F, &count, (cudaStream_t)stream);
        if (st == XTG_OK && !dry_run() && t.shape[0] != count)
            st = fail(XTG_ERR_BROADCAST, "assigned values do not match the filter's length");
    }
    if (st == XTG_OK && F.ntiles) st = filter_launch(F, t, 1, op, *dst, (cudaStream_t)stream);
    xtg_status fs = F.scratch ? scratch_free(F.scratch, (cudaStream_t)stream) : XTG_OK;
    return st != XTG_OK ? st : fs;
}

}  // extern "C"
