// xtg_blockwise.cpp — xt::blockwise reducers over arrays in device memory or
// in host memory larger than HBM (include/xtensor/reducers/
// xblockwise_reducer.hpp:15-533, xblockwise_reducer_functors.hpp:25-500).
//
// The reference reduces each block of a chunk grid with the plain reducer
// (`compute`), folds the block results of one output chunk in the grid's
// row-major order (`merge`: +=, *=, minimum / maximum, the pairwise mean /
// variance update) and finishes with `finalize` (mean / factor, sqrt,
// pow(., 1/p)).  Here the unit that moves is a slab: a range of whole block
// rows along the input's outermost dimension (largest stride).  A slab
// arrives in one of two device buffers — one DMA from pinned memory on a copy
// stream, or the threaded pinned staging ring from pageable memory — while the
// previous slab is reduced; its partial result is computed by the device
// reducers and merged into the accumulator in slab order with the reference's
// merge expressions (assign kernels).  When the slab dimension is kept, each
// slab owns a disjoint part of the output and nothing is merged.  Only the
// association of floating-point sums differs from the reference (slabs instead
// of blocks; tree sums inside a slab); integer results are identical.
#include <unistd.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <vector>

#include "xtg_plan.h"

namespace xtgh {

namespace {

struct Ex {
    xtg_expr e;
    Ex() { memset(&e, 0, sizeof e); }
    Ex& leaf(const xtg_array& a) {
        e.leaves[e.n_leaves] = a;
        xtg_node& x = e.nodes[e.n_nodes++];
        x.op = XTG_OP_LEAF;
        x.dtype = a.dtype;
        x.arg = e.n_leaves++;
        return *this;
    }
    Ex& op(int o, int arg = 0) {
        xtg_node& x = e.nodes[e.n_nodes++];
        x.op = o;
        x.dtype = -1;
        x.arg = arg;
        return *this;
    }
    Ex& f64(double v) {
        xtg_node& x = e.nodes[e.n_nodes++];
        x.op = XTG_OP_SCALAR;
        x.dtype = XTG_FLOAT64;
        x.imm.f = v;
        return *this;
    }
    Ex& scalar(int dtype, double v) {
        xtg_node& x = e.nodes[e.n_nodes++];
        x.op = XTG_OP_SCALAR;
        x.dtype = dtype;
        if (dt(dtype).is_float) x.imm.f = v;
        else if (dt(dtype).is_signed) x.imm.i = (int64_t)v;
        else x.imm.u = (uint64_t)v;
        return *this;
    }
};

enum Merge { M_ADD, M_MUL, M_MIN, M_MAX, M_VAR };
enum Fin { F_NONE, F_DIV, F_SQRT, F_POW };

struct Plan {
    int op;
    int in_dtype;
    int out_dtype;       // R: the reducer's result type
    int part_op;         // device reduction of one slab
    int part_acc;        // its acc_dtype (-1: the reducer's default)
    int part_dtype;      // its result type
    int tree;            // 0 leaf, 1 square(leaf), 2 pow(leaf, p)
    Merge merge;
    Fin fin;
};

xtg_status make_plan(const xtg_array& in, const xtg_reduce_desc* rd, Plan& P) {
    P.op = rd->op;
    P.in_dtype = in.dtype;
    P.tree = 0;
    P.part_op = rd->op;
    P.part_acc = rd->acc_dtype;
    P.fin = F_NONE;
    switch (rd->op) {
        case XTG_RED_SUM: P.merge = M_ADD; break;
        case XTG_RED_PROD: P.merge = M_MUL; break;
        case XTG_RED_AMIN: P.merge = M_MIN; P.part_acc = -1; break;
        case XTG_RED_AMAX: P.merge = M_MAX; P.part_acc = -1; break;
        case XTG_RED_MEAN: P.merge = M_ADD; P.part_op = XTG_RED_SUM; P.fin = F_DIV; break;
        case XTG_RED_VARIANCE: P.merge = M_VAR; break;
        case XTG_RED_STDDEV: P.merge = M_VAR; P.part_op = XTG_RED_VARIANCE; P.fin = F_SQRT; break;
        case XTG_RED_NORM_L0:
        case XTG_RED_NORM_L1: P.merge = M_ADD; break;
        case XTG_RED_NORM_SQ: P.merge = M_ADD; P.part_op = XTG_RED_SUM; P.tree = 1; break;
        case XTG_RED_NORM_L2: P.merge = M_ADD; P.part_op = XTG_RED_SUM; P.tree = 1; P.fin = F_SQRT; break;
        case XTG_RED_NORM_LINF: P.merge = M_MAX; break;
        case XTG_RED_NORM_LP_TO_P: P.merge = M_ADD; P.part_op = XTG_RED_SUM; P.tree = 2; break;
        case XTG_RED_NORM_LP: P.merge = M_ADD; P.part_op = XTG_RED_SUM; P.tree = 2; P.fin = F_POW; break;
        default: return fail(XTG_ERR_INVALID, "unknown reduction op");
    }
    // the result type R of the reference's functor (value_type of the plain
    // reducer; norm_type = double for the lp norms, xnorm.hpp:76-93)
    if (rd->op == XTG_RED_NORM_LP_TO_P || rd->op == XTG_RED_NORM_LP) {
        P.out_dtype = XTG_FLOAT64;
    } else {
        Ex x;
        x.leaf(in);
        xtg_reduce_desc r = *rd;
        r.n_axes = 0;
        int32_t rank;
        int64_t shape[XTG_MAX_RANK];
        XTG_TRY(xtg_reduce_shape(&x.e, &r, &rank, shape, &P.out_dtype));
    }
    // the per-block computation sums in R (sum<value_type>, mean, the norms)
    if (P.part_op == XTG_RED_SUM || rd->op == XTG_RED_VARIANCE || rd->op == XTG_RED_STDDEV || rd->op == XTG_RED_PROD)
        P.part_acc = P.out_dtype;
    P.part_dtype = P.out_dtype;
    if (rd->op == XTG_RED_AMIN || rd->op == XTG_RED_AMAX) {
        // xt::amin(input, axes, options): the block result keeps the input's type
        Ex x;
        x.leaf(in);
        xtg_reduce_desc r = *rd;
        r.acc_dtype = -1;
        r.n_axes = 0;
        int32_t rank;
        int64_t shape[XTG_MAX_RANK];
        XTG_TRY(xtg_reduce_shape(&x.e, &r, &rank, shape, &P.part_dtype));
    }
    return XTG_OK;
}

// the tree the slab partial reduces
Ex part_tree(const Plan& P, const xtg_array& slab, double p) {
    Ex x;
    x.leaf(slab);
    if (P.tree == 1) x.op(XTG_OP_SQUARE);
    if (P.tree == 2) x.f64(p).op(XTG_OP_POW);
    return x;
}

xtg_status assign_expr(Ex& x, const xtg_array& out, cudaStream_t s) { return xtg_assign(&x.e, &out, s); }

int64_t numel(const xtg_array& a) {
    int64_t n = 1;
    for (int k = 0; k < a.rank; ++k) n *= a.shape[k];
    return n;
}

xtg_array dense_like(const xtg_array& shape_of, int dtype, void* data) {
    xtg_array a = shape_of;
    a.dtype = dtype;
    a.data = data;
    int64_t s = 1;
    for (int k = a.rank - 1; k >= 0; --k) {
        a.strides[k] = s;
        s *= a.shape[k];
    }
    return a;
}

// Normalised reduced axes (the validity checks are the reducer's).
std::vector<bool> reduced_axes(const xtg_reduce_desc* rd, int rank) {
    std::vector<bool> red(rank, false);
    if (rd->n_axes < 0) {
        std::fill(red.begin(), red.end(), true);
        return red;
    }
    for (int i = 0; i < rd->n_axes && i < XTG_MAX_RANK; ++i) {
        int64_t a = rd->axes[i] < 0 ? rd->axes[i] + rank : rd->axes[i];
        if (a >= 0 && a < rank) red[a] = true;
    }
    return red;
}

enum Where { W_DEVICE, W_PINNED, W_PAGEABLE };

Where where_is(const void* p) {
    if (dry_run()) return W_PAGEABLE;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return W_PAGEABLE;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return W_DEVICE;
    if (a.type == cudaMemoryTypeHost) return W_PINNED;
    return W_PAGEABLE;
}

// Host input must be dense (no gaps) so that a slab is one byte range.
bool dense(const xtg_array& a) {
    std::vector<int> d;
    for (int k = 0; k < a.rank; ++k)
        if (a.shape[k] != 1) d.push_back(k);
    std::sort(d.begin(), d.end(), [&](int x, int y) { return a.strides[x] < a.strides[y]; });
    int64_t expect = 1;
    for (int k : d) {
        if (a.strides[k] != expect) return false;
        expect *= a.shape[k];
    }
    return true;
}

// Work spread over side streams and joined back: open() makes the side
// streams wait for everything queued on `main` so far; join() (or the
// destructor, on an early return) makes `main` wait for the side streams.
// The side streams are created once per device and kept.
struct Fork {
    cudaStream_t main = nullptr;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> ev;
    bool joined = true;
    static std::vector<cudaStream_t>& pool(int dev) {
        static std::mutex mu;
        static std::map<int, std::vector<cudaStream_t>> p;
        std::lock_guard<std::mutex> lk(mu);
        return p[dev];
    }
    xtg_status open(cudaStream_t s, int n) {
        main = s;
        int dev = 0;
        XTG_CUDA(cudaGetDevice(&dev));
        std::vector<cudaStream_t>& P = pool(dev);
        {
            static std::mutex mu;
            std::lock_guard<std::mutex> lk(mu);
            while ((int)P.size() < n) {
                cudaStream_t t;
                XTG_CUDA(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking));
                P.push_back(t);
            }
        }
        side.assign(P.begin(), P.begin() + n);
        ev.assign((size_t)n + 1, nullptr);
        for (auto& e : ev) XTG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        XTG_CUDA(cudaEventRecord(ev[0], main));
        joined = false;
        for (cudaStream_t t : side) XTG_CUDA(cudaStreamWaitEvent(t, ev[0], 0));
        return XTG_OK;
    }
    cudaStream_t stream(int i) const { return side[(size_t)i % side.size()]; }
    xtg_status join() {
        if (joined) return XTG_OK;
        joined = true;
        for (size_t i = 0; i < side.size(); ++i) {
            XTG_CUDA(cudaEventRecord(ev[i + 1], side[i]));
            XTG_CUDA(cudaStreamWaitEvent(main, ev[i + 1], 0));
        }
        return XTG_OK;
    }
    ~Fork() {
        join();
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};

struct Resources {
    cudaStream_t stream;
    std::vector<void*> scratch;
    cudaStream_t copy = nullptr;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // ready, copied[2], done[2]
    // Pageable input page-locked in place, slab by slab, for the call:
    // `regs` are consecutive ranges covering [lo, upto).
    std::vector<std::pair<uintptr_t, uintptr_t>> regs;
    uintptr_t pg = 0, lo = 0, hi = 0, upto = 0;
    bool reg_failed = false;
    // Extends the page-locked range to cover up to address `b`.
    bool cover(uintptr_t b) {
        const uintptr_t want = std::min((b + pg - 1) & ~(pg - 1), hi);
        if (want <= upto) return true;
        if (reg_failed) return false;
        if (cudaHostRegister((void*)upto, want - upto, cudaHostRegisterDefault) != cudaSuccess) {
            cudaGetLastError();
            reg_failed = true;
            return false;
        }
        regs.emplace_back(upto, want);
        upto = want;
        return true;
    }
    ~Resources() {
        if (copy) cudaStreamSynchronize(copy);  // no copy into a buffer being freed
        for (auto& r : regs) cudaHostUnregister((void*)r.first);
        for (void* p : scratch) scratch_free(p, stream);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (copy) cudaStreamDestroy(copy);
    }
    xtg_status alloc(void** p, size_t bytes) {
        XTG_TRY(scratch_alloc(p, std::max<size_t>(bytes, 16), stream));
        scratch.push_back(*p);
        return XTG_OK;
    }
};

// One block result folded into its output region: the first of a region is
// stored (converted on store when the block result type differs), later
// ones merged by the reference's merge (xblockwise_reducer_functors.hpp:
// 38-221): +=, *=, minimum, maximum, or the pairwise variance update, which
// keeps the running mean in mean_a (var_state) and the block's in mean_b.
// n_acc: elements folded into each output so far; n_b: in this block.
xtg_status fold_partial(const Plan& P, const xtg_reduce_desc& prd, const xtg_array& slab, double p, bool first,
                        const xtg_array& region, const xtg_array& part, const xtg_array& mean_a,
                        const xtg_array& mean_b, bool var_state, double n_acc, double n_b, Resources& R,
                        cudaStream_t stream) {
    Ex x = part_tree(P, slab, p);
    if (first) {
        if (P.part_dtype == P.out_dtype) {
            XTG_TRY(xtg_reduce(&x.e, &prd, &region, stream));
        } else {  // amin / amax with a wider result type: the block result converts on store
            xtg_array tmp = dense_like(region, P.part_dtype, nullptr);
            XTG_TRY(R.alloc(&tmp.data, (size_t)numel(region) * dt(P.part_dtype).size));
            XTG_TRY(xtg_reduce(&x.e, &prd, &tmp, stream));
            Ex c;
            c.leaf(tmp);
            XTG_TRY(assign_expr(c, region, stream));
        }
        if (var_state) {
            xtg_reduce_desc mrd = prd;
            mrd.op = XTG_RED_MEAN;
            Ex y;
            y.leaf(slab);
            XTG_TRY(xtg_reduce(&y.e, &mrd, &mean_a, stream));
        }
        return XTG_OK;
    }
    XTG_TRY(xtg_reduce(&x.e, &prd, &part, stream));
    Ex m;
    switch (P.merge) {
        case M_ADD: m.leaf(region).leaf(part).op(XTG_OP_ADD); break;
        case M_MUL: m.leaf(region).leaf(part).op(XTG_OP_MUL); break;
        case M_MIN: m.leaf(part).leaf(region).op(XTG_OP_MINIMUM); break;
        case M_MAX: m.leaf(part).leaf(region).op(XTG_OP_MAXIMUM); break;
        case M_VAR: {
            xtg_reduce_desc mrd = prd;
            mrd.op = XTG_RED_MEAN;
            Ex y;
            y.leaf(slab);
            XTG_TRY(xtg_reduce(&y.e, &mrd, &mean_b, stream));
            // new_mean = (n_a mean_a + n_b mean_b) / (n_a + n_b)
            // var = (n_a var_a + n_b var_b + n_a (mean_a - new_mean)^2
            //        + n_b (mean_b - new_mean)^2) / (n_a + n_b)
            // (variance_functor::merge, xblockwise_reducer_functors.hpp:195-221)
            auto new_mean = [&](Ex& e) {
                e.f64(n_acc).leaf(mean_a).op(XTG_OP_MUL).f64(n_b).leaf(mean_b).op(XTG_OP_MUL).op(XTG_OP_ADD);
                e.f64(n_acc).f64(n_b).op(XTG_OP_ADD).op(XTG_OP_DIV);
            };
            m.f64(n_acc).leaf(region).op(XTG_OP_MUL);
            m.f64(n_b).leaf(part).op(XTG_OP_MUL).op(XTG_OP_ADD);
            m.f64(n_acc).leaf(mean_a);
            new_mean(m);
            m.op(XTG_OP_SUB).op(XTG_OP_SQUARE).op(XTG_OP_MUL).op(XTG_OP_ADD);
            m.f64(n_b).leaf(mean_b);
            new_mean(m);
            m.op(XTG_OP_SUB).op(XTG_OP_SQUARE).op(XTG_OP_MUL).op(XTG_OP_ADD);
            m.f64(n_acc).f64(n_b).op(XTG_OP_ADD).op(XTG_OP_DIV);
            XTG_TRY(assign_expr(m, region, stream));
            Ex nm;
            new_mean(nm);
            XTG_TRY(assign_expr(nm, mean_a, stream));
            return XTG_OK;
        }
    }
    return assign_expr(m, region, stream);
}

xtg_status blockwise_impl(const xtg_array* in, const int64_t* block, const xtg_reduce_desc* rd, double p,
                          const xtg_array* out, cudaStream_t stream) {
    if (!in || !block || !rd || !out) return fail(XTG_ERR_INVALID, "null argument");
    if (!valid_dtype(in->dtype) || in->rank < 0 || in->rank > XTG_MAX_RANK)
        return fail(XTG_ERR_INVALID, "bad input array");
    for (int k = 0; k < in->rank; ++k) {
        if (in->shape[k] < 0) return fail(XTG_ERR_INVALID, "negative extent");
        if (block[k] < 1) return fail(XTG_ERR_INVALID, "block extents must be positive");
    }
    if (rd->has_initial) return fail(XTG_ERR_UNSUPPORTED, "blockwise reducers take no initial value");
    if (rd->ddof != 0) return fail(XTG_ERR_UNSUPPORTED, "blockwise variance takes no ddof");
    if (rd->op == XTG_RED_NORM_LP && p == 0.0)
        return fail(XTG_ERR_INVALID, "norm_lp(): p must be nonzero, use norm_l0() instead.");
    Plan P;
    XTG_TRY(make_plan(*in, rd, P));
    const int rank = in->rank;
    const std::vector<bool> red = reduced_axes(rd, rank);

    // shape checks through the plain reducer's rules
    xtg_reduce_desc prd = *rd;
    prd.op = P.part_op;
    prd.acc_dtype = P.part_acc;
    {
        Ex x = part_tree(P, *in, p);
        int32_t orank, odt;
        int64_t oshape[XTG_MAX_RANK];
        XTG_TRY(xtg_reduce_shape(&x.e, &prd, &orank, oshape, &odt));
        if (odt != P.part_dtype) return fail(XTG_ERR_INVALID, "internal: partial type");
        if (out->dtype != P.out_dtype)
            return fail(XTG_ERR_INVALID, "destination dtype " + std::to_string(out->dtype) +
                                             " differs from the result type " + std::to_string(P.out_dtype));
        bool same = out->rank == orank;
        for (int d = 0; same && d < orank; ++d) same = out->shape[d] == oshape[d];
        if (!same) return fail(XTG_ERR_SHAPE, "destination shape mismatch");
    }
    XTG_TRY(ensure_device(nullptr));
    if (numel(*out) && where_is(out->data) != W_DEVICE) return fail(XTG_ERR_INVALID, "destination is not device memory");

    Where src = numel(*in) ? where_is(in->data) : W_DEVICE;
    if (src != W_DEVICE && !dense(*in)) return fail(XTG_ERR_UNSUPPORTED, "host input must be dense");

    // slab dimension: the largest stride among extents > 1
    int k = -1;
    for (int d = 0; d < rank; ++d)
        if (in->shape[d] > 1 && (k < 0 || in->strides[d] > in->strides[k])) k = d;
    const int isz = dt(in->dtype).size;
    const int64_t rows = k < 0 ? 1 : in->shape[k];
    const int64_t row_bytes = k < 0 ? std::max<int64_t>(numel(*in), 1) * isz : in->strides[k] * isz;
    int64_t slab_rows = rows;
    if (src != W_DEVICE && k >= 0) {
        const int64_t budget = std::max<int64_t>(opt("blockwise.slab_bytes", int64_t(512) << 20), row_bytes);
        const int64_t b = block[k];
        slab_rows = b * row_bytes <= budget ? (budget / (b * row_bytes)) * b : std::max<int64_t>(1, budget / row_bytes);
        slab_rows = std::min(slab_rows, rows);
    }
    const int64_t nslabs = rows == 0 ? 1 : (rows + slab_rows - 1) / slab_rows;
    const bool slab_reduced = k >= 0 && red[k];
    // output axis of the slab dimension (when kept)
    int jout = -1;
    if (k >= 0 && !slab_reduced) {
        jout = 0;
        for (int d = 0; d < k; ++d)
            if (!red[d] || rd->keep_dims) ++jout;
    }

    Resources R;
    R.stream = stream;
    // Pageable input: each slab's pages are locked in place just before its
    // copy (the next slab's while the current one is on the link), so slabs
    // go by DMA at the link's rate instead of through the staging copy.
    // Where locking is refused (pages already registered, limits), the
    // remaining slabs take the staging ring.
    const bool lock = src == W_PAGEABLE && numel(*in) && opt("blockwise.register_host", 1);
    if (lock) {
        R.pg = (uintptr_t)sysconf(_SC_PAGESIZE);
        R.lo = R.upto = (uintptr_t)in->data & ~(R.pg - 1);
        R.hi = ((uintptr_t)in->data + (uintptr_t)(numel(*in) * dt(in->dtype).size) + R.pg - 1) & ~(R.pg - 1);
    }
    // device slab buffers
    void* dbuf[2] = {nullptr, nullptr};
    const int64_t lo_off = [&] {  // element offset of the lowest address (negative strides)
        int64_t o = 0;
        for (int d = 0; d < rank; ++d)
            if (in->strides[d] < 0 && in->shape[d] > 0) o += (in->shape[d] - 1) * in->strides[d];
        return o;
    }();
    if (src != W_DEVICE) {
        if (lo_off != 0) return fail(XTG_ERR_UNSUPPORTED, "host input with negative strides");
        const size_t sb = (size_t)(k < 0 ? row_bytes : slab_rows * row_bytes);
        XTG_TRY(R.alloc(&dbuf[0], sb));
        if (nslabs > 1) XTG_TRY(R.alloc(&dbuf[1], sb));
        for (auto& e : R.ev) XTG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        XTG_CUDA(cudaEventRecord(R.ev[0], stream));  // the buffers exist from here on
        if (src == W_PINNED || lock) {
            XTG_CUDA(cudaStreamCreateWithFlags(&R.copy, cudaStreamNonBlocking));
            XTG_CUDA(cudaStreamWaitEvent(R.copy, R.ev[0], 0));
        }
    }
    // accumulators when the slab dimension is reduced
    xtg_array part = dense_like(*out, P.part_dtype, nullptr), mean_b = dense_like(*out, P.out_dtype, nullptr);
    xtg_array mean_a = dense_like(*out, P.out_dtype, nullptr);
    const size_t on = (size_t)numel(*out);
    if (slab_reduced && nslabs > 1) {
        XTG_TRY(R.alloc(&part.data, on * dt(P.part_dtype).size));
        if (P.merge == M_VAR) XTG_TRY(R.alloc(&mean_b.data, on * dt(P.out_dtype).size));
    }
    if (P.merge == M_VAR && slab_reduced && nslabs > 1) XTG_TRY(R.alloc(&mean_a.data, on * dt(P.out_dtype).size));

    double n_acc = 0.0;
    bool used[2] = {false, false};
    for (int64_t s = 0; s < nslabs; ++s) {
        const int b = (int)(s & 1);
        const int64_t r0 = s * slab_rows, nr = std::min(slab_rows, rows - r0);
        xtg_array slab = *in;
        if (k >= 0) slab.shape[k] = nr;
        if (src == W_DEVICE) {
            if (k >= 0) slab.data = (char*)in->data + r0 * in->strides[k] * isz;
        } else {
            const size_t bytes = (size_t)(k < 0 ? (numel(*in) ? row_bytes : 0) : nr * row_bytes);
            const char* host = (const char*)in->data + (k < 0 ? 0 : r0 * row_bytes);
            slab.data = dbuf[b];
            if (bytes) {
                const uintptr_t a0 = (uintptr_t)host, a1 = a0 + bytes;
                if (src == W_PINNED || (lock && R.cover(a1))) {
                    if (used[b]) XTG_CUDA(cudaStreamWaitEvent(R.copy, R.ev[3 + b], 0));
                    if (src == W_PINNED) {
                        XTG_CUDA(cudaMemcpyAsync(dbuf[b], host, bytes, cudaMemcpyHostToDevice, R.copy));
                    } else {
                        // one copy per locked range the slab overlaps
                        for (auto& r : R.regs) {
                            const uintptr_t c0 = std::max(a0, r.first), c1 = std::min(a1, r.second);
                            if (c0 < c1)
                                XTG_CUDA(cudaMemcpyAsync((char*)dbuf[b] + (c0 - a0), (const void*)c0, c1 - c0,
                                                         cudaMemcpyHostToDevice, R.copy));
                        }
                        // lock the next slab's pages while this one is on the link
                        if (s + 1 < nslabs) R.cover(a1 + (size_t)std::min(slab_rows, rows - r0 - nr) * row_bytes);
                    }
                    XTG_CUDA(cudaEventRecord(R.ev[1 + b], R.copy));
                    XTG_CUDA(cudaStreamWaitEvent(stream, R.ev[1 + b], 0));
                } else {
                    XTG_TRY(ring_h2d(dbuf[b], host, bytes, used[b] ? R.ev[3 + b] : R.ev[0]));
                }
            }
        }
        // where this slab's partial goes
        const bool first = !slab_reduced || s == 0;
        xtg_array region = *out;
        if (jout >= 0 && nslabs > 1) {
            region.shape[jout] = nr;
            region.data = (char*)out->data + r0 * out->strides[jout] * dt(out->dtype).size;
        }
        // n_b: elements of the slab folded into each output
        double n_b = 1.0;
        for (int d = 0; d < rank; ++d)
            if (red[d]) n_b *= (double)slab.shape[d];
        XTG_TRY(fold_partial(P, prd, slab, p, first, region, part, mean_a, mean_b,
                             P.merge == M_VAR && slab_reduced && nslabs > 1, n_acc, n_b, R, stream));
        n_acc = first ? n_b : n_acc + n_b;
        if (src != W_DEVICE) {
            XTG_CUDA(cudaEventRecord(R.ev[3 + b], stream));
            used[b] = true;
        }
    }
    // finalize over the whole result
    if (P.fin != F_NONE && on) {
        Ex f;
        f.leaf(*out);
        if (P.fin == F_DIV) {
            // results /= static_cast<value_type>(factor), factor = product of the reduced extents
            int64_t factor = 1;
            for (int d = 0; d < rank; ++d)
                if (red[d]) factor *= in->shape[d];
            f.scalar(P.out_dtype, (double)factor).op(XTG_OP_DIV);
        } else if (P.fin == F_SQRT) {
            f.op(XTG_OP_SQRT);
        } else {
            f.f64(1.0 / p).op(XTG_OP_POW);
        }
        XTG_TRY(assign_expr(f, *out, stream));
    }
    if (R.copy) XTG_CUDA(cudaStreamSynchronize(R.copy));  // the host input is no longer read
    return XTG_OK;
}

// The reducer's last step over the merged block results (mean: / count,
// stddev: sqrt).
static xtg_status chunked_finish(const Plan& P, const xtg_chunked* src, const std::vector<bool>& red,
                                 const xtg_array& out, cudaStream_t stream) {
    if (P.fin == F_NONE) return XTG_OK;
    Ex f;
    f.leaf(out);
    if (P.fin == F_DIV) {
        int64_t factor = 1;
        for (int d = 0; d < src->rank; ++d)
            if (red[(size_t)d]) factor *= src->shape[d];
        f.scalar(P.out_dtype, (double)factor).op(XTG_OP_DIV);
    } else if (P.fin == F_SQRT) {
        f.op(XTG_OP_SQRT);
    }
    return assign_expr(f, out, stream);
}

// Reductions of a chunked array: each chunk's valid region (a view of its
// buffer) is one block.  The grid is walked with its reduced dims outside and
// its kept dims inside, so that every output block receives its chunks in the
// grid's row-major order and all blocks share one running element count.
xtg_status chunked_reduce_impl(const xtg_chunked* src, const xtg_reduce_desc* rd, const xtg_array* out,
                               cudaStream_t stream) {
    if (!src || !rd || !out) return fail(XTG_ERR_INVALID, "null argument");
    if (rd->has_initial) return fail(XTG_ERR_UNSUPPORTED, "chunked reductions take no initial value");
    if (rd->ddof != 0) return fail(XTG_ERR_UNSUPPORTED, "chunked variance takes no ddof");
    if (rd->op > XTG_RED_NORM_LINF) return fail(XTG_ERR_INVALID, "unknown reduction op");
    ChunkGrid G;
    XTG_TRY(chunk_grid(*src, G));
    const int rank = src->rank;
    // the whole array as a dense descriptor: types and shapes only
    xtg_array whole;
    memset(&whole, 0, sizeof whole);
    whole.dtype = src->dtype;
    whole.rank = rank;
    whole.data = G.n ? src->chunks[0] : nullptr;
    for (int d = 0; d < rank; ++d) whole.shape[d] = src->shape[d];
    whole = dense_like(whole, src->dtype, whole.data);
    Plan P;
    XTG_TRY(make_plan(whole, rd, P));
    const std::vector<bool> red = reduced_axes(rd, rank);
    xtg_reduce_desc prd = *rd;
    prd.op = P.part_op;
    prd.acc_dtype = P.part_acc;
    {
        Ex x = part_tree(P, whole, 0.0);
        int32_t orank, odt;
        int64_t oshape[XTG_MAX_RANK];
        XTG_TRY(xtg_reduce_shape(&x.e, &prd, &orank, oshape, &odt));
        if (out->dtype != P.out_dtype)
            return fail(XTG_ERR_INVALID, "destination dtype " + std::to_string(out->dtype) +
                                             " differs from the result type " + std::to_string(P.out_dtype));
        bool same = out->rank == orank;
        for (int d = 0; same && d < orank; ++d) same = out->shape[d] == oshape[d];
        if (!same) return fail(XTG_ERR_SHAPE, "destination shape mismatch");
    }
    XTG_TRY(ensure_device(nullptr));
    const int64_t on = numel(*out);
    if (G.n == 0 || on == 0) {
        // an empty reduced extent: the plain reducer's result of an empty range
        if (on == 0) return XTG_OK;
        xtg_array empty = whole;
        empty.data = out->data;  // never read: some reduced extent is 0
        Ex x;
        x.leaf(empty);
        return xtg_reduce(&x.e, rd, out, stream);
    }
    // output axis of each input dim (-1: reduced and dropped)
    int oax[XTG_MAX_RANK];
    for (int d = 0, j = 0; d < rank; ++d) oax[d] = (!red[d] || rd->keep_dims) ? j++ : -1;
    int64_t cst[XTG_MAX_RANK];
    chunk_strides(G, cst);
    std::vector<int> rdims, kdims;
    for (int d = 0; d < rank; ++d) (red[d] ? rdims : kdims).push_back(d);
    int64_t n_rcomb = 1, n_kcomb = 1;
    for (int d : rdims) n_rcomb *= G.grid[d];
    for (int d : kdims) n_kcomb *= G.grid[d];

    Resources R;
    R.stream = stream;

    // Chunks at equal distances in memory (a chunked array allocated as one
    // slab): the array is a strided array of rank 2 * rank, dims (chunk
    // index, position in the chunk) per dim, and a class of chunks with equal
    // valid extents (per dim: the full chunks, the edge chunk) is a box of
    // it.  Each class is then ONE reduction (its dims pair up: both reduced or
    // both kept), merged over the classes of the reduced dims in order.
    const int es = dt(src->dtype).size;
    const int64_t celems = [&] {
        int64_t n = 1;
        for (int d = 0; d < rank; ++d) n *= G.cs[d];
        return n;
    }();
    int64_t S = celems * es;
    bool spaced = rank >= 1 && 2 * rank <= XTG_MAX_RANK;
    if (spaced && G.n > 1) {
        S = (int64_t)((const char*)src->chunks[1] - (const char*)src->chunks[0]);
        spaced = S >= celems * es && S % es == 0;
        for (int64_t i = 2; spaced && i < G.n; ++i)
            spaced = (const char*)src->chunks[i] == (const char*)src->chunks[0] + i * S;
    }
    if (spaced) {
        struct Kind { int64_t lo, cnt, ext; };
        std::vector<Kind> kinds[XTG_MAX_RANK];
        for (int d = 0; d < rank; ++d) {
            if (G.grid[d] == 1) kinds[d] = {{0, 1, G.shape[d]}};
            else if (G.shape[d] % G.cs[d] == 0) kinds[d] = {{0, G.grid[d], G.cs[d]}};
            else kinds[d] = {{0, G.grid[d] - 1, G.cs[d]}, {G.grid[d] - 1, 1, G.shape[d] - (G.grid[d] - 1) * G.cs[d]}};
        }
        int64_t gst[XTG_MAX_RANK];
        for (int d = rank - 1, g = 1; d >= 0; --d) {
            gst[d] = g;
            g *= (int)G.grid[d];
        }
        int64_t n_rp = 1, n_kp = 1;
        for (int d : rdims) n_rp *= (int64_t)kinds[d].size();
        for (int d : kdims) n_kp *= (int64_t)kinds[d].size();
        const bool var_s = P.merge == M_VAR && n_rp > 1;
        xtg_array part = dense_like(*out, P.part_dtype, nullptr), mean_a = dense_like(*out, P.out_dtype, nullptr);
        xtg_array mean_b = dense_like(*out, P.out_dtype, nullptr);
        if (n_rp > 1) {
            XTG_TRY(R.alloc(&part.data, (size_t)on * dt(P.part_dtype).size));
            if (var_s) {
                XTG_TRY(R.alloc(&mean_a.data, (size_t)on * dt(P.out_dtype).size));
                XTG_TRY(R.alloc(&mean_b.data, (size_t)on * dt(P.out_dtype).size));
            }
        }
        // dims of the strided array: the reduced dims' chunk indexes, their
        // positions in the chunk, then (chunk index, position) per kept dim.
        // Reduced dims come first, grouped so that whole chunks merge into
        // long runs (a full reduction of a slab without gaps is one run).
        xtg_reduce_desc prd2 = prd;
        prd2.keep_dims = 0;
        prd2.n_axes = 2 * (int)rdims.size();
        for (int i = 0; i < prd2.n_axes; ++i) prd2.axes[i] = i;
        const Kind* sel[XTG_MAX_RANK];
        // the output-shaped array `a` over the kept dims' kinds: dims
        // (chunks, extent) per kept dim
        auto out_view = [&](const xtg_array& a) {
            xtg_array v = a;
            v.rank = 0;
            int64_t off = 0;
            for (int d : kdims) {
                const int64_t st = a.strides[oax[d]];
                v.shape[v.rank] = sel[d]->cnt;
                v.strides[v.rank++] = G.cs[d] * st;
                v.shape[v.rank] = sel[d]->ext;
                v.strides[v.rank++] = st;
                off += sel[d]->lo * G.cs[d] * st;
            }
            if (a.data) v.data = (char*)a.data + off * dt(a.dtype).size;
            return v;
        };
        // the strided array of the class selected in sel[]
        auto class_slab = [&]() {
            xtg_array slab = whole;
            slab.rank = 0;
            int64_t first = 0;
            for (int d = 0; d < rank; ++d) first += sel[d]->lo * gst[d];
            for (int d : rdims) {
                slab.shape[slab.rank] = sel[d]->cnt;
                slab.strides[slab.rank++] = gst[d] * (S / es);
            }
            for (int d : rdims) {
                slab.shape[slab.rank] = sel[d]->ext;
                slab.strides[slab.rank++] = cst[d];
            }
            for (int d : kdims) {
                slab.shape[slab.rank] = sel[d]->cnt;
                slab.strides[slab.rank++] = gst[d] * (S / es);
                slab.shape[slab.rank] = sel[d]->ext;
                slab.strides[slab.rank++] = cst[d];
            }
            slab.data = (void*)((const char*)src->chunks[0] + first * S);
            return slab;
        };
        // Merges other than the variance's with at most 8 reduced classes:
        // every class reduces into its own slice at once, spread over side
        // streams, then one elementwise launch per output region folds the
        // slices into it in class order (the sequential merge, one launch).
        const bool concurrent = P.merge != M_VAR && n_rp > 1 && n_rp <= 8 && P.part_dtype == P.out_dtype &&
                                opt("chunked.streams", 4) > 0 && !dry_run();
        if (concurrent) {
            const size_t psz = (size_t)on * dt(P.part_dtype).size;
            void* parts = nullptr;
            XTG_TRY(R.alloc(&parts, psz * (size_t)(n_rp - 1)));
            Fork F;
            XTG_TRY(F.open(stream, (int)std::min<int64_t>(opt("chunked.streams", 4), n_rp * n_kp)));
            int next = 0;
            for (int64_t rp = 0; rp < n_rp; ++rp) {
                int64_t q = rp;
                for (int i = (int)rdims.size() - 1; i >= 0; --i) {
                    const int d = rdims[(size_t)i];
                    sel[d] = &kinds[d][(size_t)(q % (int64_t)kinds[d].size())];
                    q /= (int64_t)kinds[d].size();
                }
                xtg_array dst = rp == 0 ? *out : dense_like(*out, P.part_dtype, (char*)parts + psz * (size_t)(rp - 1));
                for (int64_t kp = 0; kp < n_kp; ++kp) {
                    int64_t k = kp;
                    for (int i = (int)kdims.size() - 1; i >= 0; --i) {
                        const int d = kdims[(size_t)i];
                        sel[d] = &kinds[d][(size_t)(k % (int64_t)kinds[d].size())];
                        k /= (int64_t)kinds[d].size();
                    }
                    const xtg_array slab = class_slab();
                    Ex x = part_tree(P, slab, 0.0);
                    const xtg_array o = out_view(dst);
                    XTG_TRY(xtg_reduce(&x.e, &prd2, &o, F.stream(next++)));
                }
            }
            XTG_TRY(F.join());
            for (int64_t kp = 0; kp < n_kp; ++kp) {
                int64_t k = kp;
                for (int i = (int)kdims.size() - 1; i >= 0; --i) {
                    const int d = kdims[(size_t)i];
                    sel[d] = &kinds[d][(size_t)(k % (int64_t)kinds[d].size())];
                    k /= (int64_t)kinds[d].size();
                }
                const xtg_array region = out_view(*out);
                Ex m;
                if (P.merge == M_ADD || P.merge == M_MUL) {
                    m.leaf(region);
                    for (int64_t rp = 1; rp < n_rp; ++rp) {
                        m.leaf(out_view(dense_like(*out, P.part_dtype, (char*)parts + psz * (size_t)(rp - 1))));
                        m.op(P.merge == M_ADD ? XTG_OP_ADD : XTG_OP_MUL);
                    }
                } else {
                    // minimum(part_k, ... minimum(part_1, region)): the sequential merge's order
                    for (int64_t rp = n_rp - 1; rp >= 1; --rp)
                        m.leaf(out_view(dense_like(*out, P.part_dtype, (char*)parts + psz * (size_t)(rp - 1))));
                    m.leaf(region);
                    for (int64_t rp = 1; rp < n_rp; ++rp) m.op(P.merge == M_MIN ? XTG_OP_MINIMUM : XTG_OP_MAXIMUM);
                }
                XTG_TRY(assign_expr(m, region, stream));
            }
            return chunked_finish(P, src, red, *out, stream);
        }
        double n_acc2 = 0.0;
        for (int64_t rp = 0; rp < n_rp; ++rp) {
            int64_t q = rp;
            for (int i = (int)rdims.size() - 1; i >= 0; --i) {
                const int d = rdims[(size_t)i];
                sel[d] = &kinds[d][(size_t)(q % (int64_t)kinds[d].size())];
                q /= (int64_t)kinds[d].size();
            }
            double n_b = 1.0;
            for (int d : rdims) n_b *= (double)(sel[d]->cnt * sel[d]->ext);
            for (int64_t kp = 0; kp < n_kp; ++kp) {
                int64_t k = kp;
                for (int i = (int)kdims.size() - 1; i >= 0; --i) {
                    const int d = kdims[(size_t)i];
                    sel[d] = &kinds[d][(size_t)(k % (int64_t)kinds[d].size())];
                    k /= (int64_t)kinds[d].size();
                }
                xtg_array slab = class_slab();
                XTG_TRY(fold_partial(P, prd2, slab, 0.0, rp == 0, out_view(*out), out_view(part), out_view(mean_a),
                                     out_view(mean_b), var_s, n_acc2, n_b, R, stream));
            }
            n_acc2 = rp == 0 ? n_b : n_acc2 + n_b;
        }
        return chunked_finish(P, src, red, *out, stream);
    }

    const bool var_state = P.merge == M_VAR && n_rcomb > 1;
    xtg_array part = dense_like(*out, P.part_dtype, nullptr), mean_a = dense_like(*out, P.out_dtype, nullptr);
    xtg_array mean_b = dense_like(*out, P.out_dtype, nullptr);
    if (n_rcomb > 1) {
        XTG_TRY(R.alloc(&part.data, (size_t)on * dt(P.part_dtype).size));
        if (var_state) {
            XTG_TRY(R.alloc(&mean_a.data, (size_t)on * dt(P.out_dtype).size));
            XTG_TRY(R.alloc(&mean_b.data, (size_t)on * dt(P.out_dtype).size));
        }
    }
    // the view of a dense output-shaped array over one chunk's output block
    auto block_view = [&](const xtg_array& a, const int64_t* gc, const int64_t* ext) {
        xtg_array v = a;
        int64_t off = 0;
        for (int d = 0; d < rank; ++d) {
            if (oax[d] < 0) continue;
            if (red[d]) {
                v.shape[oax[d]] = 1;
            } else {
                v.shape[oax[d]] = ext[d];
                off += gc[d] * G.cs[d] * a.strides[oax[d]];
            }
        }
        if (a.data) v.data = (char*)a.data + off * dt(a.dtype).size;
        return v;
    };
    double n_acc = 0.0;
    for (int64_t rc = 0; rc < n_rcomb; ++rc) {
        int64_t gc[XTG_MAX_RANK] = {0};
        int64_t q = rc;
        for (int i = (int)rdims.size() - 1; i >= 0; --i) {
            gc[rdims[(size_t)i]] = q % G.grid[rdims[(size_t)i]];
            q /= G.grid[rdims[(size_t)i]];
        }
        double n_b = 1.0;
        for (int d : rdims) n_b *= (double)std::min(G.cs[d], G.shape[d] - gc[d] * G.cs[d]);
        for (int64_t kc = 0; kc < n_kcomb; ++kc) {
            int64_t k = kc;
            for (int i = (int)kdims.size() - 1; i >= 0; --i) {
                gc[kdims[(size_t)i]] = k % G.grid[kdims[(size_t)i]];
                k /= G.grid[kdims[(size_t)i]];
            }
            int64_t ci = 0, ext[XTG_MAX_RANK];
            for (int d = 0; d < rank; ++d) {
                ci = ci * G.grid[d] + gc[d];
                ext[d] = std::min(G.cs[d], G.shape[d] - gc[d] * G.cs[d]);
            }
            xtg_array slab = whole;
            slab.data = src->chunks[ci];
            for (int d = 0; d < rank; ++d) {
                slab.shape[d] = ext[d];
                slab.strides[d] = cst[d];
            }
            XTG_TRY(fold_partial(P, prd, slab, 0.0, rc == 0, block_view(*out, gc, ext), block_view(part, gc, ext),
                                 block_view(mean_a, gc, ext), block_view(mean_b, gc, ext), var_state, n_acc, n_b, R,
                                 stream));
        }
        n_acc = rc == 0 ? n_b : n_acc + n_b;
    }
    return chunked_finish(P, src, red, *out, stream);
}

}  // namespace

}  // namespace xtgh

using namespace xtgh;

extern "C" xtg_status xtg_chunked_reduce(const xtg_chunked* src, const xtg_reduce_desc* rd, const xtg_array* out,
                                         xtg_stream stream) {
    begin_call();
    return chunked_reduce_impl(src, rd, out, (cudaStream_t)stream);
}

extern "C" xtg_status xtg_blockwise_reduce(const xtg_array* in, const int64_t* block_shape, const xtg_reduce_desc* rd,
                                           double p, const xtg_array* out, xtg_stream stream) {
    clear_error();
    return blockwise_impl(in, block_shape, rd, p, out, (cudaStream_t)stream);
}

extern "C" xtg_status xtg_blockwise_shape(const xtg_array* in, const xtg_reduce_desc* rd, int32_t* rank,
                                          int64_t* shape, int32_t* out_dtype) {
    clear_error();
    if (!in || !rd) return fail(XTG_ERR_INVALID, "null argument");
    Plan P;
    XTG_TRY(make_plan(*in, rd, P));
    xtg_reduce_desc prd = *rd;
    prd.op = P.part_op;
    prd.acc_dtype = P.part_acc;
    Ex x = part_tree(P, *in, 2.0);
    int32_t dtp;
    XTG_TRY(xtg_reduce_shape(&x.e, &prd, rank, shape, &dtp));
    if (out_dtype) *out_dtype = P.out_dtype;
    return XTG_OK;
}
