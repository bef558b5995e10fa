// xtg_reduce.cpp — xtg_reduce / xtg_argreduce / xtg_reduce_shape.
//
// Semantics follow the reference's lazy reducer (xreducer_stepper::aggregate,
// include/xtensor/reducers/xreducer.hpp:1778-1868) and its front-ends:
//   * axes are normalised (negative -> +rank) and must be sorted, unique and in
//     bounds (xreducer.hpp:338-350, 1426-1440);
//   * the result type is decltype(reduce(init, value)) with init of type T
//     (the `sum<T>` template argument) or the value type
//     (XTENSOR_REDUCER_FUNCTION, include/xtensor/core/xmath.hpp:367-423);
//   * mean divides by (size - ddof) / n_outputs computed in integers, in
//     double (mean_division, xmath.hpp:1828-1858); variance/stddev are the
//     mean of squared deviations from the (double) mean (xmath.hpp:2082-2103);
//   * xt::initial is merged once at the end; keep_dims keeps size-1 axes.
// Execution: the reduced index space is split into a FIXED number of chunks
// that depends only on the shapes (never on the SM count), each chunk is
// reduced by one warp/CTA/thread in a fixed order, and chunks are merged in
// chunk order by a combine kernel — results are bitwise reproducible across
// runs, streams and GPUs with different SM counts.
#include <algorithm>
#include <array>
#include <cfloat>
#include <climits>
#include <cstring>
#include <string>

#include "xtg_plan.h"
#include "xtg_params.h"

namespace xtgh {


static xtg_status norm_axes(const xtg_reduce_desc* rd, int rank, std::vector<int>& axes) {
    axes.clear();
    if (rd->n_axes < 0) {
        for (int d = 0; d < rank; ++d) axes.push_back(d);
        return XTG_OK;
    }
    if (rd->n_axes > XTG_MAX_RANK) return fail(XTG_ERR_AXIS, "too many reduction axes");
    for (int i = 0; i < rd->n_axes; ++i) {
        int64_t a = rd->axes[i];
        if (a < 0) {
            a += rank;
            if (a < 0) return fail(XTG_ERR_OUT_OF_RANGE, "axis out of range");
        }
        axes.push_back((int)a);
    }
    for (size_t i = 1; i < axes.size(); ++i)
        if (axes[i] < axes[i - 1]) return fail(XTG_ERR_AXIS, "Reducing axes should be sorted.");
    for (size_t i = 1; i < axes.size(); ++i)
        if (axes[i] == axes[i - 1]) return fail(XTG_ERR_AXIS, "Reducing axes should not contain duplicates.");
    if (!axes.empty() && axes.back() > rank - 1)
        return fail(XTG_ERR_AXIS, "Axis " + std::to_string(axes.back()) + " out of bounds for reduction.");
    return XTG_OK;
}

static int big_promote(int t) {
    if (dt(t).is_float) return XTG_FLOAT64;
    return dt(t).is_signed ? XTG_INT64 : XTG_UINT64;
}
static int vcomp(int t) { return t == XTG_BFLOAT16 ? XTG_FLOAT32 : t; }

// Accumulator type of sum/prod/mean (the reference's reduce functor result).
static int acc_type(const xtg_reduce_desc* rd, int vt) {
    int init = (rd->acc_dtype >= 0 && valid_dtype(rd->acc_dtype)) ? rd->acc_dtype : vt;
    return promote(init, vt);
}

static int result_type(const xtg_reduce_desc* rd, int vt) {
    switch (rd->op) {
        case XTG_RED_SUM:
        case XTG_RED_PROD: return acc_type(rd, vt);
        case XTG_RED_AMAX:
        case XTG_RED_AMIN: return (rd->acc_dtype >= 0 && valid_dtype(rd->acc_dtype)) ? promote(rd->acc_dtype, vt) : vt;
        case XTG_RED_MEAN:
        case XTG_RED_VARIANCE:
        case XTG_RED_STDDEV:
            return (rd->acc_dtype >= 0 && valid_dtype(rd->acc_dtype)) ? rd->acc_dtype : XTG_FLOAT64;
        case XTG_RED_NORM_L0: return XTG_UINT64;
        case XTG_RED_NORM_L1:
        case XTG_RED_NORM_SQ: return big_promote(vt);
        case XTG_RED_NORM_L2: return XTG_FLOAT64;
        case XTG_RED_NORM_LINF: {
            int a = vcomp(vt);
            return (a == XTG_UINT32 || a == XTG_UINT64 || dt(a).is_float) ? a : promote(a, a);
        }
    }
    return -1;
}

struct RedShape {
    int rank = 0;                 // expression rank
    int64_t shape[XTG_MAX_RANK];  // expression shape
    std::vector<int> axes;
    bool is_red[XTG_MAX_RANK];
    int out_rank = 0;
    int64_t out_shape[XTG_MAX_RANK];
};

static xtg_status red_shape(const Tree& t, const xtg_reduce_desc* rd, bool keep_dims, RedShape& S) {
    S.rank = t.rank;
    for (int d = 0; d < t.rank; ++d) S.shape[d] = t.shape[d];
    XTG_TRY(norm_axes(rd, t.rank, S.axes));
    for (int d = 0; d < XTG_MAX_RANK; ++d) S.is_red[d] = false;
    for (int a : S.axes) S.is_red[a] = true;
    S.out_rank = 0;
    for (int d = 0; d < t.rank; ++d) {
        if (S.is_red[d]) {
            if (keep_dims) S.out_shape[S.out_rank++] = 1;
        } else {
            S.out_shape[S.out_rank++] = t.shape[d];
        }
    }
    return XTG_OK;
}

static std::string lim_lowest_f(int t, double& f, int64_t& i) {
    switch (t) {
        case XTG_FLOAT32: f = -(double)FLT_MAX; break;
        case XTG_FLOAT64: f = -DBL_MAX; break;
        case XTG_BOOL: i = 0; break;
        case XTG_INT8: i = SCHAR_MIN; break;
        case XTG_UINT8: i = 0; break;
        case XTG_INT16: i = SHRT_MIN; break;
        case XTG_UINT16: i = 0; break;
        case XTG_INT32: i = INT_MIN; break;
        case XTG_UINT32: i = 0; break;
        case XTG_INT64: i = LLONG_MIN; break;
        case XTG_UINT64: i = 0; break;
    }
    return "";
}
static void lim_max(int t, double& f, int64_t& i) {
    switch (t) {
        case XTG_FLOAT32: f = (double)FLT_MAX; break;
        case XTG_FLOAT64: f = DBL_MAX; break;
        case XTG_BOOL: i = 1; break;
        case XTG_INT8: i = SCHAR_MAX; break;
        case XTG_UINT8: i = UCHAR_MAX; break;
        case XTG_INT16: i = SHRT_MAX; break;
        case XTG_UINT16: i = USHRT_MAX; break;
        case XTG_INT32: i = INT_MAX; break;
        case XTG_UINT32: i = (int64_t)UINT_MAX; break;
        case XTG_INT64: i = LLONG_MAX; break;
        case XTG_UINT64: i = -1; break;  // all bits set
    }
}

// Stages of the column kernel's asynchronous-copy ring (0: register loads): used
// when every leaf is contiguous along the vectorised dimension with 4-, 8-
// or 16-byte vectors; 8 / leaves stages by default (the option takes up to
// 16 / leaves; at least 2), at most 4 leaves.
static int async_stages(const Tree& t, const std::vector<int>& kinds, int NL, int vec, const char* on_key, const char* stages_key) {
    if (!opt(on_key, 1) || NL < 1 || NL > 4) return 0;
    for (int l = 0; l < NL; ++l) {
        const int b = vec * dt(t.leaves[l].dtype).size;
        if (kinds[l] != 0 || !(b == 4 || b == 8 || b == 16)) return 0;
    }
    return (int)std::max<int64_t>(2, std::min<int64_t>(opt(stages_key, 8 / NL), 16 / NL));
}

static unsigned grid_cap(Kernel* k, int64_t need) {
    DeviceInfo* dev;
    ensure_device(&dev);
    int64_t cap = (int64_t)k->max_blocks_per_sm * dev->sm_count;
    return (unsigned)std::max<int64_t>(1, std::min(need, cap));
}

static bool aligned(const void* p, int64_t bytes) { return ((uintptr_t)p % (uintptr_t)bytes) == 0; }
static int kind_of(int64_t s) { return s == 1 ? 0 : (s == 0 ? 1 : 2); }

// Core launcher shared by xtg_reduce and xtg_argreduce.
//   accname  — accumulator type string; post — POST code; out_dt — output type
//   kept/red — dims of the expression shape; out strides per kept dim.
// `eout` (fused assign + reduce): the evaluated elements are also stored
// there, converted to its type (shape = the tree's shape); only the row
// strategy does that — any other plan returns XTG_ERR_UNSUPPORTED before a
// launch, and the caller evaluates in two calls instead.
static const char* kNotFusable = "fused assign + reduce: not a row reduction plan";
// One-pass moments (xtg_reduce_moments): the accumulator is xtg::AccStats and
// `outc` names the xtg::StatsOut of the four result types; only the streaming
// kernel (K13) takes it — any other plan returns XTG_ERR_UNSUPPORTED before a
// launch (with *not_fusable set) and the caller runs the four reductions.
struct StatsSpec {
    std::string outc;
    bool has_sum;  // the sum's destination is `out` (else `out` only shapes the plan)
};
static xtg_status run_reduction(const Tree& t, const std::string& accname, int post, int out_dt, const int* kept,
                                int nk, const int* red, int nr, const xtg_array& out, const int64_t* ostr_kept,
                                xtg::RedParams& p, cudaStream_t stream, const ScratchSpec* scratch,
                                const xtg_array* eout = nullptr, bool* not_fusable = nullptr,
                                const StatsSpec* stats = nullptr) {
    const int NL = (int)t.leaves.size();
    std::vector<std::array<int64_t, XTG_MAX_RANK>> full(NL);
    for (int l = 0; l < NL; ++l) leaf_bstrides(t, l, full[l].data());
    // kept group (out strides first; the fused destination's last)
    Dims K;
    K.R = nk;
    K.st.resize(1 + NL + (eout ? 1 : 0));
    for (int i = 0; i < nk; ++i) {
        K.shape[i] = t.shape[kept[i]];
        K.st[0][i] = ostr_kept[i];
        for (int l = 0; l < NL; ++l) K.st[1 + l][i] = full[l][kept[i]];
        if (eout) K.st[1 + NL][i] = eout->strides[kept[i]];
    }
    collapse(K);
    Dims Rd;
    Rd.R = nr;
    Rd.st.resize((NL > 0 ? NL : 1) + (eout ? 1 : 0));
    const int erow = NL > 0 ? NL : 1;  // the fused destination's row in Rd.st
    for (int i = 0; i < nr; ++i) {
        Rd.shape[i] = t.shape[red[i]];
        for (int l = 0; l < NL; ++l) Rd.st[l][i] = full[l][red[i]];
        if (NL == 0) Rd.st[0][i] = 0;
        if (eout) Rd.st[erow][i] = eout->strides[red[i]];
    }
    collapse(Rd);
    const int RO = K.R, RR = Rd.R;
    int64_t n_out = 1, n_red = 1;
    for (int d = 0; d < RO; ++d) n_out *= K.shape[d];
    for (int d = 0; d < RR; ++d) n_red *= Rd.shape[d];
    if (n_out == 0) return XTG_OK;
    // primary leaf: the one spanning the most elements
    int prim = -1;
    int64_t best = -1;
    for (int l = 0; l < NL; ++l) {
        int64_t n = 1;
        for (int d = 0; d < t.leaves[l].rank; ++d) n *= t.leaves[l].shape[d];
        if (n > best) {
            best = n;
            prim = l;
        }
    }
    const int64_t red_in_stride = prim >= 0 ? Rd.st[prim][RR - 1] : 1;
    const int64_t kept_in_stride = prim >= 0 ? K.st[1 + prim][RO - 1] : 1;
    bool row = true;
    if (n_out > 1 && kept_in_stride == 1 && red_in_stride != 1) row = false;
    if (n_out >= 1024 && red_in_stride == 1 && Rd.shape[RR - 1] < 32 && kept_in_stride != 1 && RR == 1) row = false;
    if (opt("reduce.force_row", 0)) row = true;
    if (eout && !row) {
        if (not_fusable) *not_fusable = true;
        return fail(XTG_ERR_UNSUPPORTED, kNotFusable);
    }

    int maxsz = 1;
    std::vector<int> kinds(NL);
    for (int l = 0; l < NL; ++l) {
        kinds[l] = kind_of(row ? Rd.st[l][RR - 1] : K.st[1 + l][RO - 1]);
        if (kinds[l] == 0) maxsz = std::max(maxsz, dt(t.leaves[l].dtype).size);
    }
    // the fused destination's vectors are as wide as its own reduction's would
    // be, so that the fold matches a later reduction of it
    if (eout) maxsz = std::max(maxsz, dt(eout->dtype).size);
    int vec = 16 / maxsz;
    auto vec_ok = [&](int v) {
        if (v == 1) return true;
        if (row ? (Rd.shape[RR - 1] % v) : (K.shape[RO - 1] % v)) return false;
        for (int l = 0; l < NL; ++l) {
            if (kinds[l] != 0) continue;
            if (!aligned(t.leaves[l].data, (int64_t)v * dt(t.leaves[l].dtype).size)) return false;
            for (int d = 0; d < RO; ++d)
                if ((row || d != RO - 1) && K.st[1 + l][d] % v) return false;
            for (int d = 0; d < RR; ++d)
                if ((!row || d != RR - 1) && Rd.st[l][d] % v) return false;
        }
        return true;
    };
    while (vec > 1 && !vec_ok(vec)) vec >>= 1;
    if (n_red == 0) vec = 1;
    // fused destination: one vector store per evaluated vector when it is
    // contiguous along the reduced run and aligned like the loads, else
    // element stores
    int es = 0;
    if (eout) {
        es = 1;
        const int64_t esz = dt(eout->dtype).size;
        if (vec > 1) {
            if (Rd.st[erow][RR - 1] != 1 || !aligned(eout->data, (int64_t)vec * esz)) es = 2;
            for (int d = 0; d < RO; ++d)
                if (K.st[1 + NL][d] % vec) es = 2;
            for (int d = 0; d + 1 < RR; ++d)
                if (Rd.st[erow][d] % vec) es = 2;
        } else if (Rd.st[erow][RR - 1] != 1) {
            es = 2;
        }
        p.eout = eout->data;
        for (int d = 0; d < RO; ++d) p.eks[d] = K.st[1 + NL][d];
        for (int d = 0; d < RR; ++d) p.ers[d] = Rd.st[erow][d];
    }

    p.n_out = n_out;
    p.n_red = n_red;
    for (int d = 0; d < RO; ++d) p.oshape[d] = K.shape[d];
    for (int d = 0; d < RR; ++d) p.rshape[d] = Rd.shape[d];
    if (row) p.rshape[RR - 1] /= vec;
    else p.oshape[RO - 1] /= vec;
    for (int d = 0; d < RO; ++d) p.ofd[d] = make_fd((uint64_t)std::max<int64_t>(p.oshape[d], 1));
    for (int d = 0; d < RR; ++d) p.rfd[d] = make_fd((uint64_t)std::max<int64_t>(p.rshape[d], 1));
    p.n_outv = row ? n_out : n_out / vec;
    p.n_redv = row ? n_red / vec : n_red;
    for (int l = 0; l < NL; ++l) {
        p.leaf[l] = t.leaves[l].data;
        for (int d = 0; d < RO; ++d) p.lks[l][d] = K.st[1 + l][d];
        for (int d = 0; d < RR; ++d) p.lrs[l][d] = Rd.st[l][d];
    }
    p.out = (stats && !stats->has_sum) ? nullptr : out.data;
    for (int d = 0; d < RO; ++d) p.ostr[d] = K.st[0][d];
    memset(&p.scal, 0, sizeof p.scal);
    for (size_t i = 0; i < t.scalars.size(); ++i) p.scal.v[i] = t.scalars[i];

    // fixed partition (depends on shapes only)
    int64_t nsplit = 1;
    if (row) {
        const int64_t target = opt("reduce.target_items", kReduceTargetItems);
        const int64_t minchunk = opt("reduce.min_chunk", 512);
        // (splitting short rows further to fill the warp slots measured
        // slower: the split combine's launch costs more than the parallelism
        // gains — C0's row sum 8.1 -> 14.3 µs)
        nsplit = std::max<int64_t>(1, std::min<int64_t>((target + n_out - 1) / n_out, p.n_redv / minchunk));
    } else {
        const int64_t target = opt("reduce.target_threads", 131072);
        const int64_t minchunk = opt("reduce.min_col_chunk", 64);
        nsplit = std::max<int64_t>(1, std::min<int64_t>((target + p.n_outv - 1) / p.n_outv, p.n_redv / minchunk));
    }
    int64_t chunk = p.n_redv > 0 ? (p.n_redv + nsplit - 1) / nsplit : 1;
    nsplit = p.n_redv > 0 ? (p.n_redv + chunk - 1) / chunk : 1;
    p.chunk = chunk;
    p.nsplit = nsplit;
    const bool big = (row ? p.n_redv : std::max(p.n_redv, p.n_outv)) > 0xFFFFFFF0ll;

    std::vector<int> order(NL), map(NL);
    for (int l = 0; l < NL; ++l) order[l] = map[l] = l;
    std::string ls = "xtg::LeafSet<";
    for (int l = 0; l < NL; ++l) {
        if (l) ls += ", ";
        ls += std::string("xtg::LeafSpec<") + dt(t.leaves[l].dtype).cname + ", " + std::to_string(kinds[l]) + ">";
    }
    ls += ">";
    const std::string tree = tree_type(t, t.root, map);
    const std::string outc = stats ? stats->outc : std::string(dt(out_dt).cname);

    // K13: a full reduction of one contiguous leaf in 16-byte vectors with a
    // double-float accumulator streams through shared memory (the same
    // vectors, order and tree as K3 with a 256-thread group, so the same bits)
    const bool dfloat = stats || accname == "xtg::AccSumC" || accname.rfind("xtg::AccMom<float", 0) == 0 ||
                        accname.rfind("xtg::AccNormC<", 0) == 0;
    const bool k13 = row && !eout && n_out == 1 && RR == 1 && NL == 1 && kinds[0] == 0 && dfloat &&
                     opt("reduce.packed", 1) && opt("reduce.stream", 1) && vec * dt(t.leaves[0].dtype).size == 16 &&
                     aligned(t.leaves[0].data, 16) && chunk >= opt("reduce.cta_chunk", 2048);
    if (stats && !k13) {
        if (not_fusable) *not_fusable = true;
        return fail(XTG_ERR_UNSUPPORTED, "one-pass moments: not a streaming plan");
    }

    void* part = nullptr;
    // split partial slots: 32 bytes, 64 for the one-pass moments' state
    const size_t part_bytes = (size_t)n_out * (size_t)nsplit * (stats ? 64 : 32);
    if (nsplit > 1) {
        if (scratch && scratch->fixed) {
            if (part_bytes > scratch->fixed_bytes)
                return fail(XTG_ERR_UNSUPPORTED, "reduction needs " + std::to_string(part_bytes) +
                                                     " bytes of scratch, more than the fixed buffer holds");
            part = scratch->fixed;
        } else {
            XTG_TRY(scratch_alloc(&part, part_bytes, stream));
        }
    }
    p.partial = part;
    // where a replayed plan patches in its fresh scratch (stream-ordered only)
    const int part_off = (part && !(scratch && scratch->fixed)) ? (int)offsetof(xtg::RedParams, partial) : -1;

    Kernel* k;
    xtg_status st;
    if (k13) {
        const int NS = (int)std::max<int64_t>(2, std::min<int64_t>(opt("reduce.stream_stages", 4), 6));
        const size_t smem = (size_t)NS * 16384;
        int* err = nullptr;
        XTG_TRY(device_error_word(&err));
        p.err = err;
        const std::string name = "xtg::k_reduce_stream<" + tree + ", " + ls + ", " + dt(t.leaves[0].dtype).cname + ", " +
                                 accname + ", " + outc + ", " + std::to_string(post) + ", " + std::to_string(vec) + ", " +
                                 std::to_string(NS) + ">";
        Kernel* k;
        st = get_kernel(name, 288, &k, smem);  // 8 consumer warps + the producer warp
        if (st == XTG_OK) st = launch(k, grid_cap(k, nsplit), 288, &p, stream, smem, part_off);
    } else if (row) {
        const int group = (chunk >= opt("reduce.cta_chunk", 2048)) ? 256 : 32;
        // (a copy ring as in the column kernel measured slower here: these
        // loops are instruction-bound once two register batches are in flight)
        std::string name = "xtg::k_reduce_row<" + tree + ", " + ls + ", " + accname + ", " + outc + ", " +
                           std::to_string(post) + ", " + std::to_string(vec) + ", " + std::to_string(RO) + ", " +
                           std::to_string(RR) + ", " + std::to_string(group) + ", " + (big ? "true" : "false") + ", " +
                           std::to_string(opt("reduce.row_unroll", 4)) +
                           (es ? ", " + std::to_string(es) + ", " + dt(eout->dtype).cname : std::string()) +
                           (opt("reduce.packed", 1) ? std::string() :
                            std::string(es ? "" : ", 0, float") + ", 0") + ">";
        st = get_kernel(name, 256, &k);
        if (st == XTG_OK) {
            int64_t items = n_out * nsplit;
            int64_t need = group == 32 ? (items + 7) / 8 : items;
            st = launch(k, grid_cap(k, need), 256, &p, stream, 0, part_off);
        }
    } else {
        const int U = (int)opt("reduce.col_unroll", 4);
        const int rs = async_stages(t, kinds, NL, vec, "reduce.col_async", "reduce.col_stages");
        const size_t ring = (size_t)rs * (size_t)NL * 256 * 16;
        std::string name = "xtg::k_reduce_col<" + tree + ", " + ls + ", " + accname + ", " + outc + ", " +
                           std::to_string(post) + ", " + std::to_string(vec) + ", " + std::to_string(RO) + ", " +
                           std::to_string(RR) + ", " + std::to_string(U) + ", " + (big ? "true" : "false") + ", " +
                           std::to_string(rs) + ">";
        st = get_kernel(name, 256, &k, ring);
        if (st == XTG_OK) {
            int64_t need = (p.n_outv * nsplit + 255) / 256;
            st = launch(k, grid_cap(k, need), 256, &p, stream, ring, part_off);
        }
    }
    if (st == XTG_OK && nsplit > 1) {
        xtg::RedParams pc = p;
        if (!row) pc.oshape[RO - 1] *= vec;  // combine decodes flat element indices
        // few splits: a thread per output merges them in order; many: a CTA
        const bool per_thread = nsplit <= opt("reduce.thread_combine_max", 64);
        std::string name = std::string(per_thread ? "xtg::k_reduce_combine_thread<" : "xtg::k_reduce_combine<") +
                           accname + ", " + outc + ", " + std::to_string(post) + ", " + std::to_string(RO) + ">";
        Kernel* kc;
        st = get_kernel(name, 256, &kc);
        if (st == XTG_OK)
            st = launch(kc, grid_cap(kc, per_thread ? (n_out + 255) / 256 : n_out), 256, &pc, stream, 0, part_off);
    }
    if (part && !(scratch && scratch->fixed)) {
        xtg_status fs = scratch_free(part, stream);
        if (st == XTG_OK) st = fs;
    }
    return st;
}

// Accumulator, post-operation and initial values of a reduction (shared by
// xtg_reduce and the batched layer).
xtg_status choose_acc(const Tree& t, const xtg_reduce_desc* rd, AccChoice& ch) {
    const int vt = t.nodes[t.root].cxx_dtype;
    const int rt = result_type(rd, vt);
    // the element compute type (after fp32 demotion)
    const int ct = vcomp(t.nodes[t.root].dtype);
    std::string acc;
    int post = 0;
    double f0 = 0;
    int64_t i0 = 0;
    const bool comp = rd->precision == XTG_PREC_COMPENSATED;
    switch (rd->op) {
        case XTG_RED_SUM:
        case XTG_RED_PROD:
        case XTG_RED_MEAN: {
            int a = acc_type(rd, vt);
            int aa = (a == XTG_FLOAT64 && ct != XTG_FLOAT64 && !t.has_f64_leaf && opt("fp32_compute", 1)) ? XTG_FLOAT32 : a;
            if (rd->op != XTG_RED_PROD && aa == XTG_FLOAT32 && comp) acc = "xtg::AccSumC";
            else acc = std::string("xtg::AccPlain<") + dt(a).cname + ", " + (rd->op == XTG_RED_PROD ? "1" : "0") + ">";
            if (rd->op == XTG_RED_PROD) f0 = 1, i0 = 1;
            if (rd->op == XTG_RED_MEAN) post = 2;
            break;
        }
        case XTG_RED_VARIANCE:
        case XTG_RED_STDDEV: {
            const char* c = (ct == XTG_FLOAT32) ? "float" : "double";
            acc = std::string("xtg::AccMom<") + c + ", " + (rd->op == XTG_RED_VARIANCE ? "1" : "2") + ">";
            break;
        }
        case XTG_RED_AMAX:
        case XTG_RED_AMIN: {
            int a = vcomp(rt);
            acc = std::string("xtg::AccSel<") + dt(a).cname + ", " + (rd->op == XTG_RED_AMAX ? "1" : "0") + ">";
            if (rd->op == XTG_RED_AMAX) lim_lowest_f(a, f0, i0);
            else lim_max(a, f0, i0);
            break;
        }
        case XTG_RED_NORM_L0: acc = "xtg::AccNorm<unsigned long long, 0>"; break;
        case XTG_RED_NORM_L1:
        case XTG_RED_NORM_SQ:
        case XTG_RED_NORM_L2: {
            int nk = rd->op == XTG_RED_NORM_L1 ? 1 : 2;
            if (ct == XTG_FLOAT32) acc = "xtg::AccNormC<" + std::to_string(nk) + ">";
            else acc = std::string("xtg::AccNorm<") + dt(big_promote(vt)).cname + ", " + std::to_string(nk) + ">";
            if (rd->op == XTG_RED_NORM_L2) post = 1;
            break;
        }
        case XTG_RED_NORM_LINF: acc = std::string("xtg::AccNorm<") + dt(vcomp(rt)).cname + ", 3>"; break;
        default: return fail(XTG_ERR_INVALID, "unknown reduction op");
    }
    ch.acc = acc;
    ch.post = post;
    ch.init_f = f0;
    ch.init_i = i0;
    ch.has_initial = rd->has_initial;
    ch.initial_f = 0;
    ch.initial_i = 0;
    ch.result_dtype = rt;
    if (rd->has_initial) {
        if (dt(rt).is_float) ch.initial_f = rd->initial.f;
        else ch.initial_i = rd->initial.i;
        if (rd->op == XTG_RED_MEAN || rd->op == XTG_RED_VARIANCE || rd->op == XTG_RED_STDDEV || rd->op >= XTG_RED_NORM_L0)
            ch.has_initial = 0;
    }
    return XTG_OK;
}

static bool out_matches(const xtg_array& out, int rank, const int64_t* shape) {
    if (out.rank != rank) return false;
    for (int d = 0; d < rank; ++d)
        if (out.shape[d] != shape[d]) return false;
    return true;
}

xtg_status reduce_impl(const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* out, cudaStream_t stream,
                       const ScratchSpec* scratch) {
    if (!rd || !out) return fail(XTG_ERR_INVALID, "null argument");
    if (rd->op < XTG_RED_SUM || rd->op > XTG_RED_NORM_LINF) return fail(XTG_ERR_INVALID, "unknown reduction op");
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside a reduction operand");
    RedShape S;
    XTG_TRY(red_shape(t, rd, rd->keep_dims != 0, S));
    const int vt = t.nodes[t.root].cxx_dtype;
    const int rt = result_type(rd, vt);
    if (out->dtype != rt)
        return fail(XTG_ERR_INVALID, "destination dtype " + std::to_string(out->dtype) + " differs from the result type " +
                                         std::to_string(rt));
    if (!out_matches(*out, S.out_rank, S.out_shape)) return fail(XTG_ERR_SHAPE, "destination shape mismatch");
    if (!out->data) return fail(XTG_ERR_INVALID, "null destination data");
    XTG_TRY(ensure_device(nullptr));

    xtg::RedParams p;
    memset(&p, 0, sizeof p);
    AccChoice ch;
    XTG_TRY(choose_acc(t, rd, ch));
    const std::string acc = ch.acc;
    const int post = ch.post;
    p.init_f = ch.init_f;
    p.init_i = ch.init_i;
    p.has_initial = ch.has_initial;
    p.initial_f = ch.initial_f;
    p.initial_i = ch.initial_i;
    // mean / variance divisor: (size - ddof) / n_outputs with integer division
    int64_t size = 1, n_out = 1;
    for (int d = 0; d < t.rank; ++d) size *= t.shape[d];
    for (int d = 0; d < t.rank; ++d)
        if (!S.is_red[d]) n_out *= t.shape[d];
    int64_t ddof = (rd->op == XTG_RED_VARIANCE || rd->op == XTG_RED_STDDEV) ? rd->ddof : 0;
    p.divisor = n_out ? (double)((size - ddof) / n_out) : 0.0;

    int kept[XTG_MAX_RANK], red[XTG_MAX_RANK], nk = 0, nr = 0;
    int64_t ostr[XTG_MAX_RANK];
    int oi = 0;
    for (int d = 0; d < t.rank; ++d) {
        if (S.is_red[d]) {
            red[nr++] = d;
            if (rd->keep_dims) ++oi;
        } else {
            kept[nk] = d;
            ostr[nk] = out->strides[oi++];
            ++nk;
        }
    }
    return run_reduction(t, acc, post, rt, kept, nk, red, nr, *out, ostr, p, stream, scratch);
}

xtg_status argreduce_impl(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, const xtg_array* out,
                          cudaStream_t stream) {
    if (!out) return fail(XTG_ERR_INVALID, "null destination");
    if (op != XTG_ARGMAX && op != XTG_ARGMIN) return fail(XTG_ERR_INVALID, "bad arg-reduction op");
    if (!valid_dtype(out->dtype) || !dt(out->dtype).is_int || out->dtype == XTG_BOOL)
        return fail(XTG_ERR_INVALID, "index destination must have an integer dtype");
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0, t));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics inside an arg-reduction operand");
    XTG_TRY(ensure_device(nullptr));
    int kept[XTG_MAX_RANK], red[XTG_MAX_RANK], nk = 0, nr = 0;
    int64_t oshape[XTG_MAX_RANK];
    int orank = 0;
    if (has_axis && t.rank > 1) {
        int64_t a = axis < 0 ? axis + t.rank : axis;
        if (a < 0 || a >= t.rank) return fail(XTG_ERR_OUT_OF_RANGE, "axis out of range");
        for (int d = 0; d < t.rank; ++d) {
            if (d == a) red[nr++] = d;
            else {
                kept[nk++] = d;
                oshape[orank++] = t.shape[d];
            }
        }
    } else {
        if (has_axis && t.rank == 1 && !(axis == 0 || axis == -1))
            return fail(XTG_ERR_OUT_OF_RANGE, "axis out of range");
        for (int d = 0; d < t.rank; ++d) red[nr++] = d;
    }
    if (!out_matches(*out, orank, oshape)) return fail(XTG_ERR_SHAPE, "index destination shape mismatch");
    int64_t n_red = 1;
    for (int i = 0; i < nr; ++i) n_red *= t.shape[red[i]];
    if (n_red == 0) return fail(XTG_ERR_INVALID, "arg-reduction over an empty axis");
    int64_t ostr[XTG_MAX_RANK];
    for (int i = 0; i < nk; ++i) ostr[i] = out->strides[i];
    const int a = vcomp(t.nodes[t.root].dtype);
    std::string acc = std::string("xtg::AccArg<") + dt(a).cname + ", " + (op == XTG_ARGMAX ? "1" : "0") + ">";
    xtg::RedParams p;
    memset(&p, 0, sizeof p);
    return run_reduction(t, acc, 0, out->dtype, kept, nk, red, nr, *out, ostr, p, stream, nullptr);
}

// Fused assign + reduce: out_e = e (xtg_assign semantics), then
// out_r = reduce(out_e) (xtg_reduce on out_e) — one pass of the row kernel
// that stores every evaluated element and folds it, when the reduction plan
// is a row plan, the tree has no row statistics and out_e shares no memory
// with the leaves; otherwise the two calls, in order.
static xtg_status assign_reduce_impl(const xtg_expr* e, const xtg_array* oute, const xtg_reduce_desc* rd,
                                     const xtg_array* outr, cudaStream_t stream) {
    if (rd->op < XTG_RED_SUM || rd->op > XTG_RED_NORM_LINF) return fail(XTG_ERR_INVALID, "unknown reduction op");
    if (!valid_dtype(oute->dtype) || oute->rank < 0 || oute->rank > XTG_MAX_RANK)
        return fail(XTG_ERR_INVALID, "bad destination descriptor");
    Tree t;
    const bool demote = opt("fp32_compute", 1) != 0 && oute->dtype != XTG_FLOAT64;
    XTG_TRY(build_tree(e, demote, t));
    // the reduction's operand is the assigned destination itself
    xtg_expr le;
    memset(&le, 0, sizeof le);
    le.n_nodes = 1;
    le.nodes[0].op = XTG_OP_LEAF;
    le.nodes[0].dtype = oute->dtype;
    le.n_leaves = 1;
    le.leaves[0] = *oute;
    // (any overlap with a leaf is excluded, in-place updates too: every split
    // of an output may read the output's first element, which another split
    // could already have overwritten)
    bool fusable = !t.n_rstats && oute->data && oute->rank == t.rank && !shares_memory(t, *oute);
    for (int d = 0; fusable && d < t.rank; ++d)
        if (oute->shape[d] != t.shape[d] || (oute->shape[d] > 1 && oute->strides[d] == 0)) fusable = false;
    if (fusable) {
        Tree te;
        XTG_TRY(build_tree(&le, false, te));
        RedShape S;
        XTG_TRY(red_shape(te, rd, rd->keep_dims != 0, S));
        const int rt = result_type(rd, te.nodes[te.root].cxx_dtype);
        if (outr->dtype != rt)
            return fail(XTG_ERR_INVALID, "destination dtype " + std::to_string(outr->dtype) +
                                             " differs from the result type " + std::to_string(rt));
        if (!out_matches(*outr, S.out_rank, S.out_shape)) return fail(XTG_ERR_SHAPE, "destination shape mismatch");
        if (!outr->data) return fail(XTG_ERR_INVALID, "null destination data");
        XTG_TRY(ensure_device(nullptr));
        xtg::RedParams p;
        memset(&p, 0, sizeof p);
        AccChoice ch;
        XTG_TRY(choose_acc(te, rd, ch));
        p.init_f = ch.init_f;
        p.init_i = ch.init_i;
        p.has_initial = ch.has_initial;
        p.initial_f = ch.initial_f;
        p.initial_i = ch.initial_i;
        int64_t size = 1, n_out = 1;
        for (int d = 0; d < te.rank; ++d) size *= te.shape[d];
        for (int d = 0; d < te.rank; ++d)
            if (!S.is_red[d]) n_out *= te.shape[d];
        const int64_t ddof = (rd->op == XTG_RED_VARIANCE || rd->op == XTG_RED_STDDEV) ? rd->ddof : 0;
        p.divisor = n_out ? (double)((size - ddof) / n_out) : 0.0;
        int kept[XTG_MAX_RANK], red[XTG_MAX_RANK], nk = 0, nr = 0;
        int64_t ostr[XTG_MAX_RANK];
        int oi = 0;
        for (int d = 0; d < te.rank; ++d) {
            if (S.is_red[d]) {
                red[nr++] = d;
                if (rd->keep_dims) ++oi;
            } else {
                kept[nk] = d;
                ostr[nk] = outr->strides[oi++];
                ++nk;
            }
        }
        bool not_fusable = false;
        const xtg_status st =
            run_reduction(t, ch.acc, ch.post, rt, kept, nk, red, nr, *outr, ostr, p, stream, nullptr, oute, &not_fusable);
        if (!not_fusable) return st;
        clear_error();
    }
    XTG_TRY(assign_guarded(t, oute, stream));
    return reduce_impl(&le, rd, outr, stream, nullptr);
}

// sum, mean, variance (ddof from rd) and norm_l2 of e over rd's axes from
// one pass when the plan streams (K13), else the four reductions in turn.
xtg_status moments_impl(const xtg_expr* e, const xtg_reduce_desc* rd0, const xtg_array* const outs[4],
                        cudaStream_t stream) {
    static const int kOps[4] = {XTG_RED_SUM, XTG_RED_MEAN, XTG_RED_VARIANCE, XTG_RED_NORM_L2};
    if (!rd0) return fail(XTG_ERR_INVALID, "null reduce descriptor");
    int first = -1;
    for (int i = 0; i < 4; ++i)
        if (outs[i] && first < 0) first = i;
    if (first < 0) return fail(XTG_ERR_INVALID, "no destination");
    xtg_reduce_desc rds[4];
    for (int i = 0; i < 4; ++i) {
        rds[i] = *rd0;
        rds[i].op = kOps[i];
        if (i != 2) rds[i].ddof = 0;
    }
    Tree t;
    XTG_TRY(build_tree(e, opt("fp32_compute", 1) != 0, t));
    bool one_pass = !t.n_rstats && !rd0->has_initial;
    RedShape S;
    if (one_pass) XTG_TRY(red_shape(t, rd0, rd0->keep_dims != 0, S));
    const int vt = t.nodes[t.root].cxx_dtype;
    int rts[4];
    for (int i = 0; one_pass && i < 4; ++i) {
        rts[i] = result_type(&rds[i], vt);
        if (!outs[i]) continue;
        if (outs[i]->dtype != rts[i])
            return fail(XTG_ERR_INVALID, "destination dtype " + std::to_string(outs[i]->dtype) +
                                             " differs from the result type " + std::to_string(rts[i]));
        if (!out_matches(*outs[i], S.out_rank, S.out_shape)) return fail(XTG_ERR_SHAPE, "destination shape mismatch");
        if (!outs[i]->data) return fail(XTG_ERR_INVALID, "null destination data");
    }
    if (one_pass) {
        AccChoice ch[4];
        for (int i = 0; i < 4; ++i) XTG_TRY(choose_acc(t, &rds[i], ch[i]));
        one_pass = ch[0].acc == "xtg::AccSumC" && ch[1].acc == "xtg::AccSumC" && ch[2].acc == "xtg::AccMom<float, 1>" &&
                   ch[3].acc == "xtg::AccNormC<2>";
    }
    if (one_pass) {
        XTG_TRY(ensure_device(nullptr));
        xtg::RedParams p;
        memset(&p, 0, sizeof p);
        int64_t size = 1, n_out = 1;
        for (int d = 0; d < t.rank; ++d) size *= t.shape[d];
        for (int d = 0; d < t.rank; ++d)
            if (!S.is_red[d]) n_out *= t.shape[d];
        p.divisor = n_out ? (double)(size / n_out) : 0.0;
        p.divisor2 = n_out ? (double)((size - rd0->ddof) / n_out) : 0.0;
        for (int i = 1; i < 4; ++i) p.out_more[i - 1] = outs[i] ? outs[i]->data : nullptr;
        const xtg_array& ref = *outs[first];
        int kept[XTG_MAX_RANK], red[XTG_MAX_RANK], nk = 0, nr = 0;
        int64_t ostr[XTG_MAX_RANK];
        int oi = 0;
        for (int d = 0; d < t.rank; ++d) {
            if (S.is_red[d]) {
                red[nr++] = d;
                if (rd0->keep_dims) ++oi;
            } else {
                kept[nk] = d;
                ostr[nk] = ref.strides[oi++];
                ++nk;
            }
        }
        StatsSpec ss;
        ss.outc = std::string("xtg::StatsOut<") + dt(rts[0]).cname + ", " + dt(rts[1]).cname + ", " + dt(rts[2]).cname +
                  ", " + dt(rts[3]).cname + ">";
        ss.has_sum = outs[0] != nullptr;
        bool not_streaming = false;
        const xtg_status st = run_reduction(t, "xtg::AccStats", 0, rts[first], kept, nk, red, nr, ref, ostr, p, stream,
                                            nullptr, nullptr, &not_streaming, &ss);
        if (!not_streaming) return st;
        clear_error();
    }
    for (int i = 0; i < 4; ++i)
        if (outs[i]) XTG_TRY(reduce_impl(e, &rds[i], outs[i], stream, nullptr));
    return XTG_OK;
}

}  // namespace xtgh

using namespace xtgh;

extern "C" {

xtg_status xtg_reduce_moments(const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* sum,
                              const xtg_array* mean, const xtg_array* variance, const xtg_array* norm_l2,
                              xtg_stream stream) {
    begin_call();
    if (!e) return fail(XTG_ERR_INVALID, "null expression");
    const xtg_array* outs[4] = {sum, mean, variance, norm_l2};
    return moments_impl(e, rd, outs, (cudaStream_t)stream);
}

xtg_status xtg_assign_reduce(const xtg_expr* e, const xtg_array* out_e, const xtg_reduce_desc* rd,
                             const xtg_array* out_r, xtg_stream stream) {
    begin_call();
    if (!e || !rd || !out_e || !out_r) return fail(XTG_ERR_INVALID, "null argument");
    return with_plan_cache(
        4, e, rd, out_r, 0, 0, 0, (cudaStream_t)stream,
        [&]() { return assign_reduce_impl(e, out_e, rd, out_r, (cudaStream_t)stream); }, out_e);
}

xtg_status xtg_reduce_shape(const xtg_expr* e, const xtg_reduce_desc* rd, int32_t* rank, int64_t* shape,
                            int32_t* out_dtype) {
    if (!rd) return fail(XTG_ERR_INVALID, "null reduce descriptor");
    if (rd->op < XTG_RED_SUM || rd->op > XTG_RED_NORM_LINF) return fail(XTG_ERR_INVALID, "unknown reduction op");
    Tree t;
    XTG_TRY(build_tree(e, false, t));
    RedShape S;
    XTG_TRY(red_shape(t, rd, rd->keep_dims != 0, S));
    if (rank) *rank = S.out_rank;
    if (shape)
        for (int d = 0; d < S.out_rank; ++d) shape[d] = S.out_shape[d];
    if (out_dtype) *out_dtype = result_type(rd, t.nodes[t.root].cxx_dtype);
    return XTG_OK;
}

xtg_status xtg_reduce_acc_dtype(const xtg_expr* e, const xtg_reduce_desc* rd, int32_t* acc) {
    if (!rd || !acc) return fail(XTG_ERR_INVALID, "null argument");
    Tree t;
    XTG_TRY(build_tree(e, false, t));
    *acc = acc_type(rd, t.nodes[t.root].cxx_dtype);
    return XTG_OK;
}

xtg_status xtg_reduce(const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* out, xtg_stream stream) {
    begin_call();
    if (!rd) return fail(XTG_ERR_INVALID, "null reduce descriptor");
    return with_plan_cache(1, e, rd, out, 0, 0, 0, (cudaStream_t)stream,
                           [&]() { return reduce_impl(e, rd, out, (cudaStream_t)stream, nullptr); });
}

xtg_status xtg_argreduce(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, const xtg_array* out,
                         xtg_stream stream) {
    begin_call();
    return with_plan_cache(2, e, nullptr, out, op, has_axis, axis, (cudaStream_t)stream,
                           [&]() { return argreduce_impl(e, op, has_axis, axis, out, (cudaStream_t)stream); });
}

}  // extern "C"
