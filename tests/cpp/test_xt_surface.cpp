// C++ call sites of xtensor compiled against the GB300 evaluator's xt::
// surface (include/xtensor/...).  The cases restate known-answer tests of
// the reference (file:line of xtensor 0.27.1's test/ directory beside each);
// the bodies are the same xtensor calls, evaluated on the GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iterator>
#include <numeric>
#include <string>
#include <vector>

#include "xtensor/chunk/xchunked_array.hpp"
#include "xtensor/chunk/xchunked_view.hpp"
#include "xtensor/containers/xarray.hpp"
#include "xtensor/containers/xtensor.hpp"
#include "xtensor/core/xmath.hpp"
#include "xtensor/core/xnoalias.hpp"
#include "xtensor/io/xnpy.hpp"
#include "xtensor/misc/xmanipulation.hpp"
#include "xtensor/misc/xsort.hpp"
#include "xtensor/reducers/xblockwise_reducer.hpp"
#include "xtensor/reducers/xnorm.hpp"
#include "xtensor/reducers/xreducer.hpp"
#include "xtensor/views/xbroadcast.hpp"
#include "xtensor/views/xview.hpp"

static int g_fail = 0, g_run = 0;
static std::vector<std::pair<std::string, std::function<void()>>>& registry() {
    static std::vector<std::pair<std::string, std::function<void()>>> r;
    return r;
}
struct Reg {
    Reg(const char* n, std::function<void()> f) { registry().emplace_back(n, f); }
};
#define TEST(A, B)                                 \
    static void A##_##B();                         \
    static Reg reg_##A##_##B(#A "." #B, A##_##B);  \
    static void A##_##B()
#define EXPECT_TRUE(c)                                                                    \
    do {                                                                                  \
        if (!(c)) {                                                                       \
            std::printf("  FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);                     \
            ++g_fail;                                                                     \
        }                                                                                 \
    } while (0)
#define EXPECT_EQ(a, b) EXPECT_TRUE((a) == (b))
#define EXPECT_NEAR(a, b, tol) EXPECT_TRUE(std::abs((double)(a) - (double)(b)) <= (tol))
#define EXPECT_THROW(stmt, ex)          \
    do {                                \
        bool caught = false;            \
        try {                           \
            stmt;                       \
        } catch (const ex&) {           \
            caught = true;              \
        }                               \
        EXPECT_TRUE(caught);            \
    } while (0)

using namespace xt;

// test_xreducer.cpp:54-82 (xreducer_features), :355-362 (sum), :475-481 (sum_all)
TEST(xreducer, sum_features) {
    xarray<double> a = ones<double>({3, 2, 4, 6, 5});
    for (std::size_t i = 0; i < 2; ++i)
        for (std::size_t j = 0; j < 6; ++j) a(1, i, 1, j, 1) = 2;
    xarray<double> res = sum(a, {1, 3});
    EXPECT_EQ(res.shape(), (std::vector<std::size_t>{3, 4, 5}));
    EXPECT_EQ((double)res(0, 0, 0), 12.0);
    EXPECT_EQ((double)res(1, 1, 1), 24.0);
    EXPECT_EQ(sum(a)(), 732.0);
}

// test_xreducer.cpp:390-397 (sum_tensor), :399-410 (single_axis_sugar)
TEST(xreducer, sum_tensor_and_sugar) {
    xtensor<double, 2> m = {{1, 2}, {3, 4}};
    xarray<double> res = xt::sum(m, {0});
    EXPECT_EQ(res.dimension(), std::size_t(1));
    EXPECT_EQ((double)res(0), 4.0);
    EXPECT_EQ((double)res(1), 6.0);
    xarray<double> r3 = xt::sum(m, {1});
    xarray<double> r4 = xt::sum(m, 1);
    EXPECT_EQ(r3, r4);
}

// test_xreducer.cpp:442-473 (sum2): negative axes and no uint8 overflow
TEST(xreducer, sum2) {
    xarray<double> u = ones<double>({2, 4});
    xarray<double> e0 = 2 * ones<double>({4});
    xarray<double> r0 = sum(u, {0});
    EXPECT_EQ(e0, r0);
    xarray<double> e1 = 4 * ones<double>({2});
    xarray<double> rm1 = sum(u, {-1});
    std::array<std::size_t, 1> a_us = {1};
    xarray<double> ru = sum(u, a_us);
    EXPECT_EQ(e1, rm1);
    EXPECT_EQ(e1, ru);
    xarray<uint8_t> c = ones<uint8_t>({1000});
    EXPECT_EQ(sum(c)(), 1000);
}

// test_xreducer.cpp:507-512 (prod<long long>)
TEST(xreducer, prod) {
    xarray<uint8_t> c = 2 * ones<uint8_t>({34});
    EXPECT_EQ(prod<long long>(c)(), 1LL << 34);
}

// test_xreducer.cpp:542-570 (mean)
TEST(xreducer, mean) {
    xtensor<double, 2> input{{-1.0, 0.0}, {1.0, 0.0}};
    EXPECT_EQ(mean(input)(), 0.0);
    xarray<double> m1 = mean(input, {1});
    EXPECT_EQ((double)m1(0), -0.5);
    EXPECT_EQ((double)m1(1), 0.5);
    xarray<uint8_t> c = {1, 2};
    EXPECT_EQ(mean(c)(), 1.5);
}

// test_xreducer.cpp:213-220 (errors), :1081-1088 (double_axis)
TEST(xreducer, errors) {
    xarray<int> a = {{1, 2, 3}, {4, 5, 6}};
    EXPECT_THROW(xarray<int> r = xt::sum(a, {1, 0}), std::runtime_error);
    EXPECT_THROW(xarray<int> r = xt::sum(a, {0, 2}), std::runtime_error);
    EXPECT_THROW(xarray<int> r = xt::sum(a, {0, 0}), std::runtime_error);
}

// test_xreducer.cpp:773-781 (chaining_reducers)
TEST(xreducer, chaining) {
    xarray<double> a = {{1., 2.}, {3., 4.}};
    auto b = a - xt::sum(a, {0});
    auto c = xt::sum(b, {0});
    EXPECT_EQ((double)c(0), -4.);
    EXPECT_EQ((double)c(1), -6.);
}

// test_xreducer.cpp:964-1018 (keep_dims, initial_value)
TEST(xreducer, keep_dims_initial) {
    xarray<double> a = arange<double>(5 * 5 * 5 * 5);
    a.reshape(std::vector<std::size_t>{5, 5, 5, 5});
    xarray<double> res = xt::sum(a, {0, 1}, xt::keep_dims | xt::evaluation_strategy::immediate);
    EXPECT_EQ(res.shape(), (std::vector<std::size_t>{1, 1, 5, 5}));
    xarray<double> r5 = xt::sum(a, {0, 2}, xt::keep_dims | initial(5));
    xarray<double> r0 = xt::sum(a, {0, 2}, xt::keep_dims);
    xarray<double> r0p5 = r0 + 5;
    EXPECT_EQ(r5, r0p5);
    xarray<double> z = xt::prod(a, {1, 2}, initial(0));
    EXPECT_EQ(xt::amax(z)(), 0.0);
}

// test_xreducer.cpp:1044-1079 (zero_shape, empty_array)
TEST(xreducer, zero_and_empty) {
    xarray<int> x = zeros<int>({0, 1});
    xarray<int> r0 = xt::sum(x, {0}, xt::keep_dims);
    EXPECT_EQ(r0.shape(), (std::vector<std::size_t>{1, 1}));
    EXPECT_EQ((int)r0(0, 0), 0);
    xarray<double> a = ones<double>({1, 2, 0, 1});
    EXPECT_TRUE(std::isnan(xt::mean(a)()));
}

// test_xnorm.cpp:97-187
TEST(xnorm, scalar_array_and_matrix) {
    xarray<int> a = -ones<int>({9});
    EXPECT_EQ(norm_l0(a)(), 9u);
    EXPECT_EQ(norm_l1(a)(), 9);
    EXPECT_EQ(norm_sq(a)(), 9);
    EXPECT_EQ(norm_l2(a)(), 3.0);
    EXPECT_EQ(norm_linf(a)(), 1);
    xarray<double> m = {{-1.0, 2.0}, {-3.0, 4.0}};
    EXPECT_EQ(norm_l1(m)(), 10.0);
    EXPECT_EQ(norm_sq(m)(), 30.0);
    EXPECT_EQ(norm_linf(m)(), 4.0);
}

// test_xsort.cpp:217-281 (argmin, argmax)
TEST(xsort, argmin_argmax) {
    xarray<double> a = {{5, 3, 1}, {4, 4, 4}};
    EXPECT_EQ(argmin(a)(), 2u);
    xarray<std::size_t> ex2 = {1, 0, 0};
    EXPECT_EQ(argmin(a, 0), ex2);
    xarray<std::size_t> ex3 = {2, 0};
    EXPECT_EQ(argmin(a, 1), ex3);
    EXPECT_EQ(argmax(a)(), 0u);
    xarray<std::size_t> mx2 = {0, 1, 1};
    EXPECT_EQ(argmax(a, 0), mx2);
    xtensor<int, 3> c = {{{1, 2, 3, 4}}, {{4, 3, 2, 1}}};
    xtensor<std::size_t, 2> ex4 = {{3}, {0}};
    EXPECT_EQ(argmax(c, 2), ex4);
    xtensor<std::size_t, 2> ex5 = {{1, 1, 0, 0}};
    EXPECT_EQ(argmax(c, 0), ex5);
}

// test_xnoalias.cpp: noalias assignment and computed assignment in place
TEST(xnoalias, assign_and_computed) {
    xarray<double> a = {{1, 2}, {3, 4}};
    xarray<double> b = {{10, 20}, {30, 40}};
    xarray<double> r = ones<double>({2, 2});
    noalias(r) = a + b;
    xarray<double> e = {{11, 22}, {33, 44}};
    EXPECT_EQ(r, e);
    noalias(r) += a;
    xarray<double> e2 = {{12, 24}, {36, 48}};
    EXPECT_EQ(r, e2);
    r = r - r(0, 0);  // `=` with aliasing: evaluated into a temporary
    EXPECT_EQ((double)r(1, 1), 36.0);
}

// test_xfunction.cpp:76-111 (broadcast shapes and broadcast_error)
TEST(xfunction, broadcasting) {
    xarray<double> a = ones<double>({3, 1, 5});
    xarray<double> b = ones<double>({4, 1});
    xarray<double> c = a + b;
    EXPECT_EQ(c.shape(), (std::vector<std::size_t>{3, 4, 5}));
    xarray<double> d = ones<double>({3, 4});
    xarray<double> f = ones<double>({5});
    EXPECT_THROW(xarray<double> g = d + f, xt::broadcast_error);
}

// test_xstrided_view.cpp:764-772 (transpose), test_strided_assign.cpp (views)
TEST(xstrided_view, transpose_and_views) {
    xarray<int> a = {{1, 2, 3}, {4, 5, 6}};
    xarray<int> t = xt::transpose(a);
    xarray<int> et = {{1, 4}, {2, 5}, {3, 6}};
    EXPECT_EQ(t, et);
    xarray<int> v = xt::view(a, xt::all(), xt::range(1, 3));
    xarray<int> ev = {{2, 3}, {5, 6}};
    EXPECT_EQ(v, ev);
    xarray<int> row = xt::view(a, 1);
    xarray<int> er = {4, 5, 6};
    EXPECT_EQ(row, er);
    auto lhs = xt::view(a, xt::all(), 0);
    lhs = xt::view(a, xt::all(), 2) * 10;
    xarray<int> ea = {{30, 2, 3}, {60, 5, 6}};
    EXPECT_EQ(a, ea);
}

// the configurations' expressions through C++ call sites
TEST(configs, c0_expression_and_row_sum) {
    const std::size_t n = 256, m = 512;
    xarray<float> A = xt::zeros<float>({n, m});
    xarray<float> b = xt::zeros<float>({m});
    {
        std::vector<float> ha(n * m), hb(m);
        for (std::size_t i = 0; i < n * m; ++i) ha[i] = (float)((int)(i * 7919 % 2001) - 1000) / 1000.0f;
        for (std::size_t j = 0; j < m; ++j) hb[j] = (float)((int)(j * 31 % 17) - 8) / 4.0f;
        A.upload(ha);
        b.upload(hb);
    }
    xarray<float> E = A * b + xt::exp(-A * A);
    xarray<float> r = xt::sum(E, {1});
    auto hE = E.to_host();
    auto hA = A.to_host();
    auto hb = b.to_host();
    double worst = 0;
    for (std::size_t i = 0; i < n * m; ++i) {
        const double ref = (double)hA[i] * hb[i % m] + std::exp(-(double)hA[i] * hA[i]);
        worst = std::max(worst, std::abs(ref - hE[i]) / (std::abs((double)hA[i] * hb[i % m]) + 1.0));
    }
    EXPECT_TRUE(worst < 4e-7);
    auto hr = r.to_host();
    for (std::size_t i = 0; i < n; ++i) {
        double s = 0, sa = 0;
        for (std::size_t j = 0; j < m; ++j) {
            s += hE[i * m + j];
            sa += std::abs(hE[i * m + j]);
        }
        EXPECT_TRUE(std::abs(hr[i] - s) <= 1e-6 * sa);
    }
}

TEST(configs, c1_normalize_transpose_amax_argmax) {
    xarray<float> x = xt::zeros<float>({8, 16, 1024});
    {
        std::vector<float> h(8 * 16 * 1024);
        for (std::size_t i = 0; i < h.size(); ++i) h[i] = (float)std::sin(0.37 * (double)i) * 3.0f;
        x.upload(h);
    }
    xarray<float> y = (x - xt::mean(x, {2}, xt::keep_dims)) / xt::sqrt(xt::variance(x, {2}, xt::keep_dims) + 1e-5);
    EXPECT_EQ(y.shape(), (std::vector<std::size_t>{8, 16, 1024}));
    xarray<double> ym = xt::mean(y, {2});
    xarray<double> yv = xt::variance(y, {2});
    auto hm = ym.to_host();
    auto hv = yv.to_host();
    for (auto v : hm) EXPECT_NEAR(v, 0.0, 1e-5);
    for (auto v : hv) EXPECT_NEAR(v, 1.0, 1e-4);
    xarray<float> t = xt::transpose(x, {2, 0, 1});
    EXPECT_EQ(t.shape(), (std::vector<std::size_t>{1024, 8, 16}));
    EXPECT_EQ((float)t(5, 3, 7), (float)x(3, 7, 5));
    xarray<float> am = xt::amax(x, {0, 2});
    EXPECT_EQ(am.shape(), (std::vector<std::size_t>{16}));
    xarray<std::size_t> ai = xt::argmax(x, 1);
    EXPECT_EQ(ai.shape(), (std::vector<std::size_t>{8, 1024}));
}

// test_xaccumulator.cpp:22-44, 147-178, 196-210 (cumsum / cumprod)
TEST(xaccumulator, one_d_dim_one_cumprod_empty) {
    xarray<int16_t> a = {int16_t(1), int16_t(2), int16_t(3), int16_t(4)};
    auto no_axis = cumsum(a);
    auto with_axis = cumsum(a, 0);
    bool promotion_works = std::is_same<typename decltype(no_axis)::value_type, int>::value;
    EXPECT_TRUE(promotion_works);
    xarray<int> expected = {1, 3, 6, 10};
    EXPECT_EQ(no_axis, expected);
    EXPECT_EQ(with_axis, expected);

    xarray<double> arr = {{5., 6., 7.}};
    xarray<double> res = cumsum(arr, 0);
    EXPECT_EQ(res, arr);

    xtensor<double, 2> t = {{1, 2, 3}, {4, 5, 6}};
    xarray<double> tres = cumsum(t, 0);
    xarray<double> texp = {{1, 2, 3}, {5, 7, 9}};
    EXPECT_EQ(tres, texp);

    xarray<long> l = {{0, 1, 2}, {3, 4, 5}, {6, 7, 8}, {9, 10, 11}};
    xarray<long> e0 = {{0, 1, 2}, {0, 4, 10}, {0, 28, 80}, {0, 280, 880}};
    xarray<long> e1 = {{0, 0, 0}, {3, 12, 60}, {6, 42, 336}, {9, 90, 990}};
    EXPECT_EQ(cumprod(l, 0), e0);
    EXPECT_EQ(cumprod(l, 1), e1);
    auto flat = cumprod(l);
    EXPECT_EQ(flat.shape(), (std::vector<std::size_t>{12}));

    xarray<double> z = ones<double>({3, 4, 0});
    EXPECT_EQ(cumsum(z).shape(), (std::vector<std::size_t>{0}));
    EXPECT_EQ(cumsum(z, 2).shape(), (std::vector<std::size_t>{3, 4, 0}));

    xarray<float> f = {{0.5f, 0.25f}, {1.f, 2.f}};
    auto fd = cumsum<double>(f, 1);
    bool is_double = std::is_same<typename decltype(fd)::value_type, double>::value;
    EXPECT_TRUE(is_double);
    bool threw = false;
    try {
        auto bad = cumsum(f, 2);
        (void)bad;
    } catch (const std::runtime_error&) {
        threw = true;
    }
    EXPECT_TRUE(threw);
}

// test_xindex_view.cpp:24-57, 68-86, 140-165 and test_xmasked_view.cpp:189-256
TEST(xviews, index_filter_masked) {
    xarray<double> e = {{0., 1., 2.}, {3., 4., 5.}, {6., 7., 8.}};
    auto v = index_view(e, {{1, 1}, {1, 2}, {2, 2}});
    EXPECT_EQ(v(0), 4.);
    v += 3;
    EXPECT_EQ((double)e(1, 1), 7.);
    v = 123.;
    EXPECT_EQ((double)e(1, 2), 123.);
    xarray<double> as = {3, 3, 3};
    v = as;
    EXPECT_EQ((double)e(2, 2), 3.);

    xarray<double> f = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    auto fv = filter(f, f > 0.);
    EXPECT_EQ(fv(0), 1.);
    fv += 2;
    EXPECT_EQ((double)f(1, 1), 3.);
    fv += xarray<double>{1, 2, 3};
    EXPECT_EQ((double)f(1, 1), 5.);
    EXPECT_EQ((double)f(2, 2), 6.);

    xarray<double> a = {{1, 5, 3}, {4, 5, 6}};
    filtration(a, a >= 5.) += 2;
    xarray<double> ea = {{1, 7, 3}, {4, 7, 8}};
    EXPECT_EQ(a, ea);
    xarray<double> a2 = {{1, 5, 3}, {4, 5, 6}};
    const xarray<double> b = {{1, 5, 3}, {4, 5, 6}};
    filter(a2, a2 > 3.) += filter(b, b > 3.);
    xarray<double> ea2 = {{1, 10, 3}, {8, 10, 12}};
    EXPECT_EQ(a2, ea2);

    xarray<double> data = {{1., -2., 3.}, {4., 5., -6.}, {7., 8., -9.}};
    xarray<bool> mask = {{true, true, true}, {true, false, false}, {true, false, true}};
    masked_view(data, mask) = 3.65;
    xarray<double> e1 = {{3.65, 3.65, 3.65}, {3.65, 5., -6.}, {3.65, 8., 3.65}};
    EXPECT_EQ(data, e1);
    masked_view(data, mask) += 3.;
    xarray<double> e2 = {{6.65, 6.65, 6.65}, {6.65, 5., -6.}, {6.65, 8., 6.65}};
    EXPECT_EQ(data, e2);
}

// test_xnpy.cpp:39-83 (load), 125-170 (dump) on the reference's fixtures
static std::string npy_file(const std::string& stem) {
    const char* d = std::getenv("XTG_NPY_DIR");
    return std::string(d ? d : "tests/golden/npy") + "/" + stem + ".le.npy";
}
static std::string read_bytes(const std::string& name) {
    std::ifstream f(name, std::ios::binary);
    return std::string((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}
TEST(xnpy, load_dump) {
    xarray<double> darr = {{{0.29731723, 0.04380157, 0.94748308}, {0.85020643, 0.52958618, 0.0598172},
                            {0.77253259, 0.47564231, 0.70274005}},
                           {{0.85998447, 0.61160158, 0.44432939}, {0.25506765, 0.97420976, 0.15455842},
                            {0.05873659, 0.66191764, 0.01448838}},
                           {{0.175919, 0.13850365, 0.94059426}, {0.79941809, 0.5124432, 0.51364796},
                            {0.25721979, 0.41608858, 0.06255319}}};
    xarray<bool> barr = {{{0, 0, 1}, {1, 1, 0}, {1, 0, 1}}, {{1, 1, 0}, {0, 1, 0}, {0, 1, 0}},
                         {{0, 0, 1}, {1, 1, 1}, {0, 0, 0}}};
    xarray<int> iarr1d = {3, 4, 5, 6, 7};

    auto darr_loaded = load_npy<double>(npy_file("double"));
    EXPECT_TRUE(allclose(darr, darr_loaded));
    std::ifstream dstream(npy_file("double"), std::ios::binary);
    auto darr_loaded_stream = load_npy<double>(dstream);
    EXPECT_TRUE(allclose(darr, darr_loaded_stream));
    auto barr_loaded = load_npy<bool>(npy_file("bool"));
    EXPECT_EQ(barr, barr_loaded);
    auto dfarr_loaded = load_npy<double, layout_type::column_major>(npy_file("double_fortran"));
    EXPECT_TRUE(allclose(darr, dfarr_loaded));
    auto iarr1d_loaded = load_npy<int>(npy_file("int"));
    EXPECT_EQ(iarr1d, iarr1d_loaded);
    EXPECT_THROW(load_npy<float>(npy_file("double")), std::runtime_error);
    EXPECT_THROW((load_npy<double, layout_type::row_major>(npy_file("double_fortran"))), std::runtime_error);
    EXPECT_THROW(load_npy<double>(std::string("no/such/file.npy")), std::runtime_error);

    EXPECT_TRUE(dump_npy(barr) == read_bytes(npy_file("bool")));
    xtensor<uint64_t, 1> ularr = {12ul, 14ul, 16ul, 18ul, 1234321ul};
    const std::string fn = "test_dump_1.npy";
    dump_npy(fn, ularr);
    auto ularrcpy = load_npy<uint64_t>(fn);
    EXPECT_TRUE(allclose(ularr, ularrcpy));
    EXPECT_TRUE(read_bytes(fn) == read_bytes(npy_file("unsignedlong")));
    EXPECT_TRUE(dump_npy(ularr) == read_bytes(npy_file("unsignedlong")));
    std::remove(fn.c_str());
    // an expression is evaluated before it is written
    auto twice = load_npy<double>([&] {
        std::ofstream o("test_dump_2.npy", std::ios::binary);
        o << dump_npy(darr * 2.);
        o.close();
        return std::string("test_dump_2.npy");
    }());
    EXPECT_TRUE(allclose(twice, darr * 2.));
    std::remove("test_dump_2.npy");
}

// test_xblockwise_reducer.cpp:95-140: blockwise::op equals the plain reducer
template <class BR, class PR> static void check_blockwise(BR reducer, PR should_reducer, bool close) {
    auto should = xt::eval(should_reducer);
    EXPECT_EQ(reducer.dimension(), should.dimension());
    EXPECT_TRUE(std::vector<std::size_t>(reducer.shape().begin(), reducer.shape().end()) ==
                std::vector<std::size_t>(should.shape().begin(), should.shape().end()));
    auto result = xarray<typename BR::value_type>::from_shape(reducer.shape());
    reducer.assign_to(result);
    if (close) EXPECT_TRUE(allclose(result, should));
    else EXPECT_TRUE(result == should);
}
TEST(xreducer, explicit_all_axes_to_fresh_container) {
    xarray<int> a = {{1, 2}, {3, 4}};
    xarray<int> s = xt::sum(a, std::vector<std::size_t>{0, 1});  // 0-d, built from the expression
    EXPECT_EQ(s.dimension(), 0u);
    EXPECT_EQ(s(), 10);
}
TEST(xblockwise_reducer, test_values) {
    const std::vector<std::size_t> shape = {21, 10, 5}, chunk_shape = {5, 4, 2};
    std::vector<int> h(21 * 10 * 5);
    std::iota(h.begin(), h.end(), -5);
    for (std::size_t i = 0; i < h.size(); ++i)
        if (i % 2) h[i] += 10;
    xarray<int> input_exp(shape);
    input_exp.upload(h);
    const std::vector<std::vector<std::size_t>> axes_vec = {{0}, {1}, {2}, {0, 1}, {0, 2}, {0, 1, 2}};
    for (const auto& axes : axes_vec) {
        check_blockwise(blockwise::sum(input_exp, chunk_shape, axes, keep_dims), xt::sum(input_exp, axes, keep_dims), false);
        check_blockwise(blockwise::prod(input_exp, chunk_shape, axes), xt::prod(input_exp, axes), false);
        check_blockwise(blockwise::amin(input_exp, chunk_shape, axes, keep_dims), xt::amin(input_exp, axes, keep_dims), false);
        check_blockwise(blockwise::amax(input_exp, chunk_shape, axes), xt::amax(input_exp, axes), false);
        check_blockwise(blockwise::mean(input_exp, chunk_shape, axes, keep_dims), xt::mean(input_exp, axes, keep_dims), false);
        check_blockwise(blockwise::variance(input_exp, chunk_shape, axes), xt::variance(input_exp, axes), true);
        check_blockwise(blockwise::stddev(input_exp, chunk_shape, axes, keep_dims), xt::stddev(input_exp, axes, keep_dims), true);
        check_blockwise(blockwise::norm_l1(input_exp, chunk_shape, axes), xt::norm_l1(input_exp, axes), false);
        check_blockwise(blockwise::norm_linf(input_exp, chunk_shape, axes, keep_dims), xt::norm_linf(input_exp, axes, keep_dims), false);
        check_blockwise(blockwise::norm_lp(input_exp, chunk_shape, 2.0, axes), xt::norm_l2(input_exp, axes), true);
        // the same input from host memory, streamed by slabs
        check_blockwise(blockwise::sum(adapt_host(h.data(), shape), chunk_shape, axes), xt::sum(input_exp, axes), false);
    }
}

// ---- chunked arrays (test_xchunked_array.cpp, test_xchunked_view.cpp)
TEST(xchunked_array, indexed_access) {  // test_xchunked_array.cpp:20-44
    auto a = chunked_array<double>({10, 10, 10}, {2, 3, 4});
    std::vector<size_t> idx = {3, 9, 8};
    double val = 1.;
    a[idx] = val;
    EXPECT_EQ((double)a[idx], val);
    EXPECT_EQ((double)a(3, 9, 8), val);
    val = 2.;
    a(3, 9, 8) = val;
    EXPECT_EQ((double)a(3, 9, 8), val);
    EXPECT_EQ((double)a[idx], val);
}

TEST(xchunked_array, assign_expression) {  // test_xchunked_array.cpp:46-126
    std::vector<size_t> shape1 = {2, 2, 2};
    std::vector<size_t> chunk_shape1 = {2, 3, 4};
    auto a1 = chunked_array<double>(shape1, chunk_shape1);
    double val = 3.;
    a1 = broadcast(val, a1.shape());
    for (double v : a1.to_host()) EXPECT_EQ(v, val);
    std::vector<size_t> shape2 = {32, 10, 10};
    auto a2 = chunked_array<double>(shape2, chunk_shape1);
    a2 = broadcast(val, a2.shape());
    for (double v : a2.to_host()) EXPECT_EQ(v, val);
    a2 += a2;
    for (double v : a2.to_host()) EXPECT_EQ(v, 2. * val);
    a2 += 2.;
    for (double v : a2.to_host()) EXPECT_EQ(v, 2. * val + 2.);
    xarray<double> a3{{1., 2., 3.}, {4., 5., 6.}, {7., 8., 9.}};
    EXPECT_EQ(is_chunked(a3), false);
    std::vector<size_t> chunk_shape4 = {2, 2};
    auto a4 = chunked_array(a3, chunk_shape4);
    EXPECT_EQ(is_chunked(a4), true);
    double i = 1.;
    for (double v : a4.to_host()) {
        EXPECT_EQ(v, i);
        i += 1.;
    }
    auto a5 = xchunked_array<double>(a4, a4.chunk_shape());
    EXPECT_EQ(is_chunked(a5), true);
    for (auto v : a5.chunk_shape()) EXPECT_EQ(v, 2u);
    auto a6 = chunked_array(a3);
    EXPECT_EQ(is_chunked(a6), true);
    for (auto v : a6.chunk_shape()) EXPECT_EQ(v, 3u);
    std::vector<size_t> shape3 = {3, 3};
    std::vector<size_t> chunk_shape3 = {1, 2};
    auto a7 = chunked_array<double>(shape3, chunk_shape3);
    a7 = a3;
    for (auto it = a7.chunks().begin(); it != a7.chunks().end(); ++it)
        EXPECT_TRUE(std::vector<size_t>(it->shape().begin(), it->shape().end()) == chunk_shape3);
    EXPECT_TRUE(a7 == a3);
}

TEST(xchunked_array, noalias) {  // test_xchunked_array.cpp:128-137
    std::vector<std::size_t> shape = {10, 10, 10};
    std::vector<std::size_t> chunk_shape = {2, 2, 2};
    auto a = chunked_array<double>(shape, chunk_shape);
    xt::xarray<double> b = arange(1000).reshape({10, 10, 10});
    noalias(a) = b;
    EXPECT_TRUE(a == b);
}

TEST(xchunked_array, chunk_iterator) {  // test_xchunked_array.cpp:139-168
    std::vector<std::size_t> shape = {10, 10, 10};
    std::vector<std::size_t> chunk_shape = {2, 2, 2};
    auto a = chunked_array<double>(shape, chunk_shape);
    xt::xarray<double> b = arange(1000).reshape({10, 10, 10});
    noalias(a) = b;
    auto it = a.chunk_begin();
    auto cit = a.chunk_cbegin();
    for (size_t i = 0; i < 5; ++i)
        for (size_t j = 0; j < 5; ++j)
            for (size_t k = 0; k < 5; ++k) {
                EXPECT_EQ((*it).flat(0), (double)a(2 * i, 2 * j, 2 * k));
                EXPECT_EQ((*cit).flat(0), (double)a(2 * i, 2 * j, 2 * k));
                ++it;
                ++cit;
            }
    it = a.chunk_begin();
    std::advance(it, 2);
    EXPECT_EQ((*it).flat(0), (double)a(0, 0, 4));
}

TEST(xchunked_array, reducers) {  // xt::sum / amax / mean of a chunked array
    xt::xarray<double> b = arange(1000).reshape({10, 10, 10});
    auto a = chunked_array(b, std::vector<std::size_t>{3, 4, 5});
    EXPECT_TRUE(xarray<double>(xt::sum(a, {1})) == xarray<double>(xt::sum(b, {1})));
    EXPECT_TRUE(xarray<double>(xt::amax(a, {0, 2})) == xarray<double>(xt::amax(b, {0, 2})));
    EXPECT_EQ(xt::sum(a)(), 499500.);
    EXPECT_NEAR(xt::mean(a)(), 499.5, 1e-12);
}

TEST(xchunked_view, iterate) {  // test_xchunked_view.cpp:16-31
    std::vector<std::size_t> shape = {3, 4};
    std::vector<std::size_t> chunk_shape = {1, 2};
    xarray<double> a(shape);
    std::size_t chunk_nb = 0;
    auto chunked_view = xchunked_view<xarray<double>>(a, chunk_shape);
    for (auto it = chunked_view.chunk_begin(); it != chunked_view.chunk_end(); it++) chunk_nb++;
    std::size_t expected_chunk_nb = (shape[0] / chunk_shape[0]) * (shape[1] / chunk_shape[1]);
    EXPECT_EQ(chunk_nb, expected_chunk_nb);
}

TEST(xchunked_view, assign) {  // test_xchunked_view.cpp:33-45
    std::vector<std::size_t> shape = {3, 4};
    std::vector<std::size_t> chunk_shape = {1, 2};
    xarray<double> a(shape);
    std::vector<double> data = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
    a.upload(data);
    xarray<double> b(shape);
    as_chunked(b, chunk_shape) = a;
    EXPECT_TRUE(a == b);
}

TEST(xchunked_view, assign_chunked_array) {  // test_xchunked_view.cpp:47-61
    std::vector<std::size_t> shape = {10, 10, 10};
    std::vector<std::size_t> chunk_shape = {2, 3, 4};
    auto a = chunked_array<double>(shape, chunk_shape);
    xarray<double> b(shape);
    auto ref = arange(1000).reshape({10, 10, 10});
    as_chunked(a, chunk_shape) = ref;
    as_chunked(b, chunk_shape) = a;
    EXPECT_TRUE(ref == a);
    EXPECT_TRUE(ref == b);
}

int main() {
    for (auto& t : registry()) {
        const int before = g_fail;
        ++g_run;
        try {
            t.second();
        } catch (const std::exception& e) {
            std::printf("  FAIL %s: exception %s\n", t.first.c_str(), e.what());
            ++g_fail;
        }
        std::printf("%s %s\n", g_fail == before ? "[ OK ]" : "[FAIL]", t.first.c_str());
    }
    std::printf("%d tests, %d failed checks\n", g_run, g_fail);
    return g_fail ? 1 : 0;
}
