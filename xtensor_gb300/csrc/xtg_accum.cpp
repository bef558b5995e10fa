// xtg_accum.cpp — accumulators: xt::cumsum / cumprod / nancumsum / nancumprod.
//
// The reference (include/xtensor/reducers/xaccumulator.hpp:202-310) converts
// the expression into the accumulation type and folds it sequentially along
// one axis, or over the row-major flattening into a 1-D result.  Here the
// expression tree is evaluated inside the scan kernels (no temporary) over an
// (outer, axis, inner) space:
//   inner > 1           -> K9a k_scan_col   (a thread walks the axis)
//   inner == 1, many rows or short rows
//                       -> K9b k_scan_rows  (a warp folds 32 rows in order)
//   a few long rows     -> K9c segmented    (segment totals, their prefix in
//                                            order, each segment rescanned)
// When the outer or inner dims cannot be merged into one (a flattened
// transposed view, for instance) the expression is first evaluated into a
// contiguous temporary of the accumulation type — which is what the
// reference's `result_type res = e` does for every call.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "xtg_plan.h"

namespace xtgh {

namespace {

int kind_of_s(int64_t s) { return s == 1 ? 0 : (s == 0 ? 1 : 2); }
bool aligned_to(const void* p, int64_t bytes) { return ((uintptr_t)p % (uintptr_t)bytes) == 0; }

std::string leafset_s(const Tree& t, const std::vector<int>& kinds) {
    std::string s = "xtg::LeafSet<";
    for (size_t i = 0; i < t.leaves.size(); ++i) {
        if (i) s += ", ";
        s += std::string("xtg::LeafSpec<") + dt(t.leaves[i].dtype).cname + ", " + std::to_string(kinds[i]) + ">";
    }
    return s + ">";
}

unsigned grid_of(Kernel* k, int64_t need) {
    DeviceInfo* dev;
    ensure_device(&dev);
    const int64_t cap = (int64_t)k->max_blocks_per_sm * dev->sm_count;
    return (unsigned)std::max<int64_t>(1, std::min(need, cap));
}

// Merge a run of dims [d0, d1) of D (every array) into at most one dim.
// Returns false when they do not collapse.
bool merge_run(const Dims& D, int d0, int d1, int64_t& n, std::vector<int64_t>& st) {
    Dims S;
    S.R = 0;
    S.st.resize(D.st.size());
    for (int d = d0; d < d1; ++d) {
        S.shape[S.R] = D.shape[d];
        for (size_t a = 0; a < D.st.size(); ++a) S.st[a][S.R] = D.st[a][d];
        ++S.R;
    }
    collapse(S);
    st.assign(D.st.size(), 0);
    if (S.R == 0) {
        n = 1;
        return true;
    }
    if (S.R > 1) return false;
    n = S.shape[0];
    for (size_t a = 0; a < D.st.size(); ++a) st[a] = S.st[a][0];
    return true;
}

int acc_result_type(const Tree& t, int acc_dtype) {
    const int vt = t.nodes[t.root].cxx_dtype;
    return promote(acc_dtype >= 0 ? acc_dtype : vt, vt);
}

struct AccPlan {
    int R = 0;
    int64_t shape[XTG_MAX_RANK];
    int ax = -1;  // -1: flattened
};

xtg_status acc_plan(const Tree& t, int32_t has_axis, int64_t axis, AccPlan& P) {
    P.R = t.rank;
    for (int d = 0; d < t.rank; ++d) P.shape[d] = t.shape[d];
    if (!has_axis) return XTG_OK;
    const int64_t a = axis < 0 ? axis + t.rank : axis;
    if (a < 0 || a >= t.rank) return fail(XTG_ERR_AXIS, "Axis larger than expression dimension in accumulator.");
    P.ax = (int)a;
    return XTG_OK;
}

xtg_status scan_launch(const Tree& t, int rt, int op, const AccPlan& P, const xtg_array& out, cudaStream_t stream);

xtg_status accumulate_impl(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                           const xtg_array* out, cudaStream_t stream) {
    if (!out) return fail(XTG_ERR_INVALID, "null destination");
    if (op < XTG_ACC_CUMSUM || op > XTG_ACC_NANCUMPROD) return fail(XTG_ERR_INVALID, "bad accumulator op");
    if (acc_dtype >= XTG_NUM_DTYPES) return fail(XTG_ERR_INVALID, "bad accumulation dtype");
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0 && out->dtype != XTG_FLOAT64, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside an accumulator operand");
    XTG_TRY(ensure_device(nullptr));
    const int rt = acc_result_type(t, acc_dtype);
    if (out->dtype != rt) return fail(XTG_ERR_INVALID, "destination dtype is not the accumulation type");
    AccPlan P;
    XTG_TRY(acc_plan(t, has_axis, axis, P));
    int64_t total = 1;
    for (int d = 0; d < P.R; ++d) total *= P.shape[d];
    if (P.ax < 0) {
        if (out->rank != 1 || out->shape[0] != total) return fail(XTG_ERR_SHAPE, "flattened accumulation shape");
    } else {
        if (out->rank != P.R) return fail(XTG_ERR_SHAPE, "accumulation shape");
        for (int d = 0; d < P.R; ++d)
            if (out->shape[d] != P.shape[d]) return fail(XTG_ERR_SHAPE, "accumulation shape");
    }
    if (total == 0) return XTG_OK;
    if (!out->data) return fail(XTG_ERR_INVALID, "null destination data");
    return scan_launch(t, rt, op, P, *out, stream);
}

xtg_status scan_launch(const Tree& t, int rt, int op, const AccPlan& P, const xtg_array& out, cudaStream_t stream) {
    const int NL = (int)t.leaves.size();
    const int R = std::max(P.R, 1);
    // the space over the expression's shape; the destination's strides over
    // it (flattened: row-major linear index times the 1-D stride)
    Dims D;
    D.R = R;
    D.st.resize(1 + NL);
    for (int d = 0; d < R; ++d) D.shape[d] = P.R ? P.shape[d] : 1;
    if (P.ax >= 0) {
        for (int d = 0; d < R; ++d) D.st[0][d] = out.strides[d];
    } else {
        int64_t m = out.strides[0];
        for (int d = R - 1; d >= 0; --d) {
            D.st[0][d] = D.shape[d] == 1 ? 0 : m;
            m *= D.shape[d];
        }
    }
    for (int l = 0; l < NL; ++l) {
        if (P.R) bstrides_to(t.leaves[l], R, D.shape, D.st[1 + l].data());
        else D.st[1 + l][0] = 0;
    }
    int64_t n_outer = 1, len = 1, n_inner = 1;
    std::vector<int64_t> so, sa, si;
    bool ok;
    if (P.ax < 0) {
        ok = merge_run(D, 0, R, len, sa);
        so.assign(1 + NL, 0);
        si.assign(1 + NL, 0);
    } else {
        ok = merge_run(D, 0, P.ax, n_outer, so) && merge_run(D, P.ax + 1, R, n_inner, si);
        len = D.shape[P.ax];
        sa.resize(1 + NL);
        for (int a = 0; a <= NL; ++a) sa[a] = D.st[a][P.ax];
    }
    if (!ok || NL == 0) {
        // evaluate into a contiguous temporary of the accumulation type and
        // scan that (the reference's `result_type res = e`)
        const int64_t total = [&] {
            int64_t n = 1;
            for (int d = 0; d < P.R; ++d) n *= P.shape[d];
            return n;
        }();
        if (recorder()) recorder()->nocache = true;  // the temporary's address is baked into the launches
        void* tmp = nullptr;
        XTG_TRY(scratch_alloc(&tmp, (size_t)total * dt(rt).size + 16, stream));
        xtg_array ta;
        memset(&ta, 0, sizeof ta);
        ta.data = tmp;
        ta.dtype = rt;
        ta.rank = P.R;
        int64_t m = 1;
        for (int d = P.R - 1; d >= 0; --d) {
            ta.shape[d] = P.shape[d];
            ta.strides[d] = m;
            m *= P.shape[d];
        }
        xtg_status st = assign_tree(t, &ta, stream);
        if (st == XTG_OK) {
            xtg_expr le;
            memset(&le, 0, sizeof le);
            le.n_nodes = 1;
            le.nodes[0].op = XTG_OP_LEAF;
            le.nodes[0].arg = 0;
            le.nodes[0].dtype = rt;
            le.n_leaves = 1;
            le.leaves[0] = ta;
            Tree t2;
            st = build_tree(&le, false, t2);
            if (st == XTG_OK) st = scan_launch(t2, rt, op, P, out, stream);
        }
        xtg_status fs = scratch_free(tmp, stream);
        return st != XTG_OK ? st : fs;
    }

    xtg::ScanParams p;
    memset(&p, 0, sizeof p);
    p.n_outer = n_outer;
    p.len = len;
    p.n_inner = n_inner;
    for (int l = 0; l < NL; ++l) {
        p.leaf[l] = t.leaves[l].data;
        p.lso[l] = so[1 + l];
        p.lsa[l] = sa[1 + l];
        p.lsi[l] = si[1 + l];
    }
    p.out = out.data;
    p.oso = so[0];
    p.osa = sa[0];
    p.osi = si[0];
    for (size_t i = 0; i < t.scalars.size(); ++i) p.scal.v[i] = t.scalars[i];
    std::vector<int> map(NL);
    for (int l = 0; l < NL; ++l) map[l] = l;
    const std::string tree = tree_type(t, t.root, map);
    const std::string rts = dt(rt).cname;
    const std::string ops = std::to_string(op);

    if (n_inner > 1) {
        // K9a: VEC adjacent inner positions per thread when every leaf is
        // contiguous or broadcast along the inner dim and the destination
        // contiguous
        int maxsz = dt(rt).size;
        for (int l = 0; l < NL; ++l)
            if (p.lsi[l] == 1) maxsz = std::max(maxsz, dt(t.leaves[l].dtype).size);
        int vec = std::max(1, 16 / maxsz);
        auto vec_ok = [&](int v) {
            if (v == 1) return true;
            if (p.osi != 1 || n_inner % v || (p.oso % v) || (p.osa % v)) return false;
            if (!aligned_to(out.data, (int64_t)v * dt(rt).size)) return false;
            for (int l = 0; l < NL; ++l) {
                if (p.lsi[l] != 1 && p.lsi[l] != 0) return false;
                if (p.lsi[l] == 1 && ((p.lso[l] % v) || (p.lsa[l] % v) ||
                                      !aligned_to(p.leaf[l], (int64_t)v * dt(t.leaves[l].dtype).size)))
                    return false;
            }
            return true;
        };
        while (vec > 1 && !vec_ok(vec)) vec >>= 1;
        std::vector<int> kinds(NL);
        for (int l = 0; l < NL; ++l) kinds[l] = kind_of_s(p.lsi[l]);
        const int okind = p.osi == 1 ? 0 : 2;
        std::string name = "xtg::k_scan_col<" + tree + ", " + leafset_s(t, kinds) + ", " + rts + ", " + ops + ", " +
                           std::to_string(vec) + ", " + std::to_string(okind) + ", 4>";
        Kernel* k;
        XTG_TRY(get_kernel(name, 256, &k));
        const int64_t work = n_outer * (n_inner / vec);
        return launch(k, grid_of(k, (work + 255) / 256), 256, &p, stream);
    }

    std::vector<int> kinds(NL, 2);
    const std::string ls = leafset_s(t, kinds);
    int64_t strategy = opt("scan.strategy", 0);  // 0 auto, 1 rows, 2 tiles
    if (strategy == 0) strategy = (n_outer >= 4096 || len <= 2048) ? 1 : 2;
    if (strategy == 1) {
        // VEC adjacent columns per lane when the rows allow 16-byte accesses
        int maxsz = dt(rt).size;
        for (int l = 0; l < NL; ++l)
            if (p.lsa[l] == 1) maxsz = std::max(maxsz, dt(t.leaves[l].dtype).size);
        int vec = std::max(1, 16 / maxsz);
        if (vec * dt(rt).size > 16) vec = 16 / dt(rt).size;
        auto vec_ok = [&](int v) {
            if (v == 1) return true;
            if (len % v || p.osa != 1 || p.oso % v || !aligned_to(out.data, (int64_t)v * dt(rt).size)) return false;
            for (int l = 0; l < NL; ++l)
                if (p.lsa[l] == 1 && (p.lso[l] % v || !aligned_to(p.leaf[l], (int64_t)v * dt(t.leaves[l].dtype).size)))
                    return false;
            return true;
        };
        while (vec > 1 && !vec_ok(vec)) vec >>= 1;
        std::vector<int> rk(NL);
        for (int l = 0; l < NL; ++l) rk[l] = vec > 1 ? kind_of_s(p.lsa[l]) : 2;
        // a plain contiguous operand of the accumulation type goes into the
        // shared-memory tile by asynchronous copies (all 32 rows in flight)
        const int vb = vec * dt(rt).size;
        const bool raw = opt("scan.async", 1) && NL == 1 && t.nodes[t.root].op == XTG_OP_LEAF &&
                         t.leaves[0].dtype == rt && p.lsa[0] == 1 && (vb == 4 || vb == 8 || vb == 16);
        std::string name = "xtg::k_scan_rows<" + tree + ", " + leafset_s(t, rk) + ", " + rts + ", " + ops + ", " +
                           std::to_string(vec) + ", " + (raw ? "true" : "false") + ">";
        Kernel* k;
        XTG_TRY(get_kernel(name, 64, &k));
        const int64_t groups = (n_outer + 31) / 32;
        return launch(k, grid_of(k, (groups + 1) / 2), 64, &p, stream);
    }
    // K9c: segmented reduce-then-scan, one warp per segment: segments of
    // whole 512-element units, about one segment per resident warp of the
    // apply pass (so every warp of its single wave has one segment of equal
    // length)
    DeviceInfo* dev;
    XTG_TRY(ensure_device(&dev));
    const int rsz = dt(rt).size;
    // 16-byte register loads / stores when every leaf is contiguous or
    // broadcast along the rows and the destination contiguous, all aligned
    int sv = std::min(8, 16 / rsz);  // at most the 8 elements a lane holds in the register form
    for (int l = 0; l < NL; ++l)
        if (p.lsa[l] == 1) sv = std::min(sv, 16 / dt(t.leaves[l].dtype).size);
    auto sv_ok = [&](int v) {
        if (v == 1) return true;
        if (p.osa != 1 || p.oso % v || !aligned_to(out.data, (int64_t)v * rsz)) return false;
        for (int l = 0; l < NL; ++l) {
            if (p.lsa[l] != 0 && p.lsa[l] != 1) return false;
            if (p.lsa[l] == 1 && (p.lso[l] % v || !aligned_to(p.leaf[l], (int64_t)v * dt(t.leaves[l].dtype).size)))
                return false;
        }
        return true;
    };
    while (sv > 1 && !sv_ok(sv)) sv >>= 1;
    std::vector<int> sk(NL);
    for (int l = 0; l < NL; ++l) sk[l] = sv > 1 ? kind_of_s(p.lsa[l]) : 2;
    const std::string sls = leafset_s(t, sk), svs = std::to_string(sv);
    // A plain contiguous operand of the accumulation type (4 or 8 bytes,
    // 16-byte vectors): the apply pass streams warp tiles of 32 x 16 elements
    // through a per-warp cp.async ring of NS stages; for float64 pass A keeps
    // the lanes' tile totals for it (CS).  Otherwise warp tiles of 32 x 8
    // in registers.
    const bool raw = opt("scan.async", 1) && NL == 1 && t.nodes[t.root].op == XTG_OP_LEAF &&
                     t.leaves[0].dtype == rt && p.lsa[0] == 1 && (rsz == 4 || rsz == 8) && sv * rsz == 16;
    const int ns = raw ? (int)std::max<int64_t>(2, std::min<int64_t>(8, opt("scan.seg_stages", 3))) : 0;
    const int ipt_c = raw ? 16 : 8;
    const bool cs = raw && rt == XTG_FLOAT64 && opt("scan.lane_totals", 1);
    const int ipt_a = raw || rsz <= 4 ? 16 : 8;  // streamed operands: pass A's tiles are pass C's
    // lane chains: two for streamed float64, with or without CS, so that
    // both give the same bits (four cost more FP64 adds than they hide:
    // 1.11 against 0.90 ms on 2^27 elements)
    const int nch = raw && rt == XTG_FLOAT64 ? 2 : 1;
    // stages x warps x (warp tile + the lanes' folds)
    const size_t ring = (size_t)ns * 8 * ((size_t)32 * ipt_c * rsz + (cs ? (size_t)32 * nch * rsz : 0));
    const std::string tail_a = ", " + svs + ", " + std::to_string(ipt_a) + ", " + (cs ? "true" : "false") + ", " +
                               std::to_string(nch) + ">";
    const std::string tail_c = ", " + svs + ", " + std::to_string(ns) + ", " + std::to_string(ipt_c) + ", " +
                               (cs ? "true" : "false") + ", " + std::to_string(nch) + ">";
    Kernel *ka, *kb, *kc;
    XTG_TRY(get_kernel("xtg::k_scan_seg_reduce<" + tree + ", " + sls + ", " + rts + ", " + ops + tail_a, 256, &ka));
    XTG_TRY(get_kernel("xtg::k_scan_seg_apply<" + tree + ", " + sls + ", " + rts + ", " + ops + tail_c, 256, &kc, ring));
    const int64_t unit = 512;
    const int64_t nunits = (len + unit - 1) / unit;
    const int64_t warps = (int64_t)kc->max_blocks_per_sm * dev->sm_count * 8;
    const int64_t target = std::max<int64_t>(1, warps / std::max<int64_t>(1, n_outer));
    const int64_t seg_units = std::max<int64_t>(1, (nunits + target - 1) / target);
    const int64_t nseg = (nunits + seg_units - 1) / seg_units;
    if (seg_units >= (1ll << 32) || nseg >= (1ll << 30)) return fail(XTG_ERR_UNSUPPORTED, "scan too long");
    // pass B stages a row's segment totals in shared memory
    const size_t seg_smem = ((size_t)nseg * 16 + 15) & ~(size_t)15;
    if (seg_smem > 200 * 1024) return fail(XTG_ERR_UNSUPPORTED, "scan: too many segments per row");
    XTG_TRY(get_kernel("xtg::k_scan_seg_offsets<" + rts + ", " + ops + ">", 256, &kb, seg_smem));
    p.ntiles = nunits;
    p.n_inner = (nseg << 32) | seg_units;
    // one scratch block: the segment states, then (CS) one value per lane
    // of every warp tile of every row
    const size_t agg_bytes = ((size_t)n_outer * (size_t)nseg * 16 + 255) & ~(size_t)255;
    const size_t cs_bytes = cs ? (size_t)n_outer * (size_t)nunits * 32 * nch * rsz : 0;
    p.csum_off = cs ? (int64_t)agg_bytes : 0;
    void* agg = nullptr;
    XTG_TRY(scratch_alloc(&agg, agg_bytes + cs_bytes, stream));
    p.agg = agg;
    const int agg_off = (int)offsetof(xtg::ScanParams, agg);
    const int64_t blocks = (n_outer * nseg + 7) / 8;  // eight warps per block
    xtg_status st = launch(ka, grid_of(ka, blocks), 256, &p, stream, 0, agg_off);
    if (st == XTG_OK) st = launch(kb, grid_of(kb, n_outer), 256, &p, stream, seg_smem, agg_off);
    if (st == XTG_OK) st = launch(kc, grid_of(kc, blocks), 256, &p, stream, ring, agg_off);
    xtg_status fs = scratch_free(agg, stream);
    return st != XTG_OK ? st : fs;
}

}  // namespace

xtg_status accumulate_call(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                           const xtg_array* out, cudaStream_t stream) {
    return accumulate_impl(e, op, has_axis, axis, acc_dtype, out, stream);
}

}  // namespace xtgh

using namespace xtgh;

extern "C" {

xtg_status xtg_accumulate_shape(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                                int32_t* rank, int64_t* shape, int32_t* dtype) {
    if (op < XTG_ACC_CUMSUM || op > XTG_ACC_NANCUMPROD) return fail(XTG_ERR_INVALID, "bad accumulator op");
    if (acc_dtype >= XTG_NUM_DTYPES) return fail(XTG_ERR_INVALID, "bad accumulation dtype");
    Tree t;
    XTG_TRY(build_tree(e, false, t));
    AccPlan P;
    XTG_TRY(acc_plan(t, has_axis, axis, P));
    if (P.ax < 0) {
        int64_t n = 1;
        for (int d = 0; d < P.R; ++d) n *= P.shape[d];
        if (rank) *rank = 1;
        if (shape) shape[0] = n;
    } else {
        if (rank) *rank = P.R;
        if (shape)
            for (int d = 0; d < P.R; ++d) shape[d] = P.shape[d];
    }
    if (dtype) *dtype = acc_result_type(t, acc_dtype);
    return XTG_OK;
}

xtg_status xtg_accumulate(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                          const xtg_array* out, xtg_stream stream) {
    begin_call();
    return with_plan_cache(3, e, nullptr, out, op | ((acc_dtype + 1) << 8), has_axis, axis, (cudaStream_t)stream,
                           [&]() { return accumulate_impl(e, op, has_axis, axis, acc_dtype, out, (cudaStream_t)stream); });
}

}  // extern "C"
