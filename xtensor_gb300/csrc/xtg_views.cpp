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
//  * filter(e, cond) and filtration(dst, cond) take P = the inclusive count
//    of cond in row-major order (a cumsum of the condition as int64, the
//    accumulator kernels), then element i is selected when P[i] > P[i-1] and
//    lands at P[i] - 1 — the order of argwhere (xindex_view.hpp:821-826).
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

// the inclusive count of cond over `shape` (row-major) into a temporary
xtg_status positions(const xtg_expr* cond, int rank, const int64_t* shape, void** P, int64_t* total,
                     cudaStream_t stream) {
    Tree tc;
    XTG_TRY(build_tree(cond, false, tc));
    if (tc.rank != rank) return fail(XTG_ERR_SHAPE, "condition shape differs from the filtered expression's");
    for (int d = 0; d < rank; ++d)
        if (tc.shape[d] != shape[d]) return fail(XTG_ERR_SHAPE, "condition shape differs from the filtered expression's");
    int64_t n = 1;
    for (int d = 0; d < rank; ++d) n *= shape[d];
    *total = n;
    xtg_expr c64;
    memset(&c64, 0, sizeof c64);
    XTG_TRY(append_expr(c64, cond));
    {
        // cast(cond != 0, int64)
        xtg_node z;
        memset(&z, 0, sizeof z);
        z.op = XTG_OP_SCALAR;
        z.dtype = XTG_INT32;
        z.imm.i = 0;
        if (c64.n_nodes + 3 > XTG_MAX_NODES) return fail(XTG_ERR_UNSUPPORTED, "condition expression is too large");
        c64.nodes[c64.n_nodes++] = z;
        XTG_TRY(push_op(c64, XTG_OP_NE));
        XTG_TRY(push_op(c64, XTG_OP_CAST, XTG_INT64));
    }
    XTG_TRY(scratch_alloc(P, (size_t)std::max<int64_t>(n, 1) * 8, stream));
    xtg_array pa;
    memset(&pa, 0, sizeof pa);
    pa.data = *P;
    pa.dtype = XTG_INT64;
    pa.rank = 1;
    pa.shape[0] = n;
    pa.strides[0] = 1;
    xtg_status st = n ? accumulate_call(&c64, XTG_ACC_CUMSUM, 0, 0, XTG_INT64, &pa, stream) : XTG_OK;
    if (st != XTG_OK) scratch_free(*P, stream);
    return st;
}

xtg_status count_of(void* P, int64_t n, int64_t* count, cudaStream_t stream) {
    if (n == 0 || dry_run()) {
        *count = 0;
        return XTG_OK;
    }
    long long c = 0;
    XTG_CUDA(cudaMemcpyAsync(&c, (const long long*)P + (n - 1), 8, cudaMemcpyDeviceToHost, stream));
    XTG_CUDA(cudaStreamSynchronize(stream));
    *count = c;
    return XTG_OK;
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
        if (mode == 0 || mode == 2) {
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
    void* P = nullptr;
    int64_t n = 0;
    XTG_TRY(positions(cond, tc.rank, tc.shape, &P, &n, (cudaStream_t)stream));
    xtg_status st = count_of(P, n, count, (cudaStream_t)stream);
    xtg_status fs = scratch_free(P, (cudaStream_t)stream);
    return st != XTG_OK ? st : fs;
}

xtg_status xtg_filter(const xtg_expr* e, const xtg_expr* cond, const xtg_array* out, xtg_stream stream) {
    begin_call();
    if (!out) return fail(XTG_ERR_INVALID, "null destination");
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0 && out->dtype != XTG_FLOAT64, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside a filter");
    if (t.rank < 1) return fail(XTG_ERR_INVALID, "filter of a 0-d expression");
    void* P = nullptr;
    int64_t n = 0, count = 0;
    XTG_TRY(positions(cond, t.rank, t.shape, &P, &n, (cudaStream_t)stream));
    xtg_status st = count_of(P, n, &count, (cudaStream_t)stream);
    if (st == XTG_OK && !dry_run() && (out->rank != 1 || out->shape[0] != count))
        st = fail(XTG_ERR_SHAPE, "filter result must be 1-D of xtg_filter_count elements");
    if (st == XTG_OK && n) st = launch_indexed(t, 2, 0, t.rank, t.shape, (const long long*)P, n, *out, (cudaStream_t)stream);
    xtg_status fs = scratch_free(P, (cudaStream_t)stream);
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
    void* P = nullptr;
    int64_t n = 0, count = 0;
    XTG_TRY(positions(cond, dst->rank, dst->shape, &P, &n, (cudaStream_t)stream));
    xtg_status st = XTG_OK;
    if (t.rank == 1 && t.shape[0] != 1) {
        st = count_of(P, n, &count, (cudaStream_t)stream);
        if (st == XTG_OK && !dry_run() && t.shape[0] != count)
            st = fail(XTG_ERR_BROADCAST, "assigned values do not match the filter's length");
    }
    if (st == XTG_OK && n)
        st = launch_indexed(t, 3, op, dst->rank, dst->shape, (const long long*)P, n, *dst, (cudaStream_t)stream);
    xtg_status fs = scratch_free(P, (cudaStream_t)stream);
    return st != XTG_OK ? st : fs;
}

}  // extern "C"
