// nt2_demos.cpp -- NT2's hot-path demos written against nt2/table.hpp and run
// by libnt2gpu.  The expressions are spelled as in NT2's demo sources:
//   demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59   (bs_demo)
//   demo/sdot/nt2/sdot_nt2.cpp:37                         (sdot)
//   demo/saxpy/nt2/saxpy_nt2.cpp:41                       (saxpy)
//   demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:30-32                (rgb2yuv, as one tie)
//   demo/sigmadelta/nt2/sigmadelta_nt2.cpp:38-57          (sigmadelta, as one tie)
// plus the textbook call+put of the fused Black-Scholes workload (bs).
//
// usage: nt2_demos lower
//        nt2_demos bs|bs_host|bs_demo|saxpy|rgb2yuv DIR N
//        nt2_demos sdot DIR N
//        nt2_demos threads|streams DIR N   (reductions from two host threads / on two streams)
//        nt2_demos fold|fold_expr DIR M N
//        nt2_demos gen DIR N
//        nt2_demos sigmadelta DIR PIXELS FRAMES
// Inputs and outputs are raw little-endian arrays DIR/<name>.bin.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "nt2/table.hpp"

using dtable = nt2::table<float, nt2::device_>;
using htable = nt2::table<float>;
using u8table = nt2::table<std::uint8_t, nt2::device_>;

template <class T> static std::vector<T> read_bin(const std::string &path, std::size_t n)
{
    std::vector<T> v(n);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <class T> static void write_bin(const std::string &path, const std::vector<T> &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
}

template <class Tab> static Tab load(const std::string &path, std::size_t n)
{
    using T = typename Tab::value_type;
    nt2::table<T> h(nt2::of_size(n));
    auto v = read_bin<T>(path, n);
    std::memcpy(h.data(), v.data(), n * sizeof(T));
    Tab t;
    t = h;
    return t;
}

template <class Tab> static void save(const std::string &path, const Tab &t)
{
    using T = typename Tab::value_type;
    nt2::table<T> h;
    h = t;
    write_bin(path, std::vector<T>(h.data(), h.data() + h.numel()));
}

// textbook call + put as one fused assignment
template <class Tab> static void blackscholes(Tab &C, Tab &P, const Tab &S, const Tab &K, const Tab &T, float r,
                                              float sigma)
{
    auto sq = nt2::sqrt(T);
    auto d1 = (nt2::log(S / K) + nt2::fma(nt2::sqr(sigma), 0.5f, r) * T) / (sigma * sq);
    auto d2 = nt2::fnms(sigma, sq, d1);
    auto e = K * nt2::exp(-r * T);
    nt2::tie(C, P) = nt2::tie(nt2::fnms(e, nt2::normcdf(d2), S * nt2::normcdf(d1)),
                              nt2::fnms(S, nt2::normcdf(-d1), e * nt2::normcdf(-d2)));
}

static int lower_only()
{
    const std::size_t n = 64;
    htable S(nt2::of_size(n)), K(nt2::of_size(n)), T(nt2::of_size(n)), C(nt2::of_size(n)), P(nt2::of_size(n));
    {
        const float r = 0.02f, sigma = 0.30f;
        auto sq = nt2::sqrt(T);
        auto d1 = (nt2::log(S / K) + nt2::fma(nt2::sqr(sigma), 0.5f, r) * T) / (sigma * sq);
        auto d2 = nt2::fnms(sigma, sq, d1);
        auto e = K * nt2::exp(-r * T);
        std::printf("bs %s\n", nt2::tie(C, P).explain(nt2::tie(nt2::fnms(e, nt2::normcdf(d2), S * nt2::normcdf(d1)),
                                                           nt2::fnms(S, nt2::normcdf(-d1), e * nt2::normcdf(-d2))))
                                   .c_str());
    }
    {
        htable Sa(nt2::of_size(n)), Xa(nt2::of_size(n)), Ta(nt2::of_size(n)), ra(nt2::of_size(n)),
            va(nt2::of_size(n)), R(nt2::of_size(n));
        auto da = nt2::sqrt(Ta);
        auto d1 = nt2::log(Sa / Xa) + (nt2::fma(nt2::sqr(va), 0.5f, ra) * Ta) / (va * da);
        auto d2 = nt2::fnms(va, da, d1);
        std::printf("bs_demo %s\n",
                    nt2::tie(R).explain(nt2::tie(nt2::fnms(Xa * nt2::exp(-ra * Ta), nt2::fastnormcdf(d2),
                                                           Sa * nt2::fastnormcdf(d1))))
                        .c_str());
    }
    {
        htable X(nt2::of_size(n)), Y(nt2::of_size(n));
        std::printf("saxpy %s\n", nt2::tie(Y).explain(nt2::tie(2.5f * X + Y)).c_str());
    }
    {
        htable r(nt2::of_size(n)), g(nt2::of_size(n)), b(nt2::of_size(n)), y(nt2::of_size(n)), u(nt2::of_size(n)),
            v(nt2::of_size(n));
        std::printf("rgb2yuv %s\n", nt2::tie(y, u, v)
                                        .explain(nt2::tie(0.299f * r + 0.587f * g + 0.114f * b, 0.492f * (b - y),
                                                          0.877f * (r - y)))
                                        .c_str());
    }
    {
        nt2::table<std::uint8_t> fr(nt2::of_size(n)), bkg(nt2::of_size(n)), var(nt2::of_size(n)),
            out(nt2::of_size(n));
        auto diff = nt2::max(bkg, fr) - nt2::min(bkg, fr);
        auto mul = nt2::adds(nt2::adds(diff, diff), diff);
        std::printf("sigmadelta %s\n",
                    nt2::tie(bkg, var, out)
                        .explain(nt2::tie(nt2::selinc(bkg < fr, nt2::seldec(bkg > fr, bkg)),
                                          nt2::if_else(diff != std::uint8_t(0),
                                                       nt2::selinc(var < mul, nt2::seldec(var > mul, var)), var),
                                          nt2::if_zero_else_one(diff < var)))
                        .c_str());
    }
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s lower | bs|bs_host|bs_demo|saxpy|rgb2yuv|sdot|threads|streams DIR N | "
                             "fold|fold_expr DIR M N | sigmadelta DIR PIXELS FRAMES\n",
                     argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    if (mode == "lower") return lower_only();
    if (argc < 4) return 2;
    const std::string dir = std::string(argv[2]) + "/";
    const std::size_t n = std::strtoull(argv[3], nullptr, 10);
    if (const char *p = std::getenv("NT2G_PRECISION")) nt2::options().precision = std::atoi(p);
    try {
        if (mode == "bs") {
            auto S = load<dtable>(dir + "S.bin", n), K = load<dtable>(dir + "K.bin", n), T = load<dtable>(dir + "T.bin", n);
            dtable C(nt2::of_size(n)), P(nt2::of_size(n));
            blackscholes(C, P, S, K, T, 0.02f, 0.30f);
            save(dir + "call.bin", C);
            save(dir + "put.bin", P);
        } else if (mode == "bs_host") {  // host tables: staged to the device and back
            auto S = load<htable>(dir + "S.bin", n), K = load<htable>(dir + "K.bin", n), T = load<htable>(dir + "T.bin", n);
            htable C(nt2::of_size(n)), P(nt2::of_size(n));
            blackscholes(C, P, S, K, T, 0.02f, 0.30f);
            save(dir + "call.bin", C);
            save(dir + "put.bin", P);
        } else if (mode == "bs_demo") {
            auto Sa = load<dtable>(dir + "S.bin", n), Xa = load<dtable>(dir + "K.bin", n),
                 Ta = load<dtable>(dir + "T.bin", n), ra = load<dtable>(dir + "r.bin", n),
                 va = load<dtable>(dir + "v.bin", n);
            dtable R(nt2::of_size(n));
            // as in the demo, da/d1/d2 are materialised tables
            dtable da, d1, d2;
            da = nt2::sqrt(Ta);
            d1 = nt2::log(Sa / Xa) + (nt2::fma(nt2::sqr(va), 0.5f, ra) * Ta) / (va * da);
            d2 = nt2::fnms(va, da, d1);
            R = nt2::fnms(Xa * nt2::exp(-ra * Ta), nt2::fastnormcdf(d2), Sa * nt2::fastnormcdf(d1));
            save(dir + "R.bin", R);
        } else if (mode == "saxpy") {
            auto X = load<dtable>(dir + "x.bin", n), Y = load<dtable>(dir + "y.bin", n);
            const float alpha = read_bin<float>(dir + "alpha.bin", 1)[0];
            Y = alpha * X + Y;
            save(dir + "y_out.bin", Y);
        } else if (mode == "rgb2yuv") {
            auto r = load<dtable>(dir + "r.bin", n), g = load<dtable>(dir + "g.bin", n), b = load<dtable>(dir + "b.bin", n);
            dtable y(nt2::of_size(n)), u(nt2::of_size(n)), v(nt2::of_size(n));
            nt2::tie(y, u, v) = nt2::tie(0.299f * r + 0.587f * g + 0.114f * b, 0.492f * (b - y), 0.877f * (r - y));
            save(dir + "y.bin", y);
            save(dir + "u.bin", u);
            save(dir + "v.bin", v);
        } else if (mode == "sdot") {
            auto X = load<dtable>(dir + "x.bin", n), Y = load<dtable>(dir + "y.bin", n);
            std::printf("globalsum %.17g\nsum64 %.17g\ndot %.9g\nsum %.9g\n", (double)nt2::globalsum(X * Y),
                        nt2::sum64(X * Y), (double)nt2::dot(X, Y), (double)nt2::sum(X));
            // a sum of a general expression is folded in one pass (no temporary)
            std::printf("sum_expr %.17g\n", nt2::sum64(nt2::sqr(X) + Y));
        } else if (mode == "fold_expr") {
            // reductions of expressions over an M x N pair of tables (N = argv[4]), in one pass each
            const std::size_t cols = std::strtoull(argv[4], nullptr, 10);
            nt2::table<float> ha(nt2::of_size(n, cols)), hb(nt2::of_size(n, cols));
            auto va = read_bin<float>(dir + "a.bin", n * cols), vb = read_bin<float>(dir + "b.bin", n * cols);
            std::memcpy(ha.data(), va.data(), va.size() * sizeof(float));
            std::memcpy(hb.data(), vb.data(), vb.size() * sizeof(float));
            dtable A, B;
            A = ha;
            B = hb;
            save(dir + "sumabs1.bin", nt2::sum(nt2::abs(A - B), 1));
            save(dir + "maxexp2.bin", nt2::maximum(nt2::exp(A) - B, 2));
            save(dir + "var1.bin", nt2::var(A * B + 1.0f, 0, 1));
            std::int64_t imax = 0;
            const float gmax = nt2::globalmax(A * B + 1.0f, imax);
            std::printf("globalmax %.9g %lld\nglobalsum %.17g\nglobalmean %.9g\n", (double)gmax, (long long)imax,
                        nt2::sum64(nt2::exp(A) * B), (double)nt2::globalmean(nt2::abs(A - B)));
        } else if (mode == "threads") {
            // two host threads, each on its own stream with its own tables, reduce concurrently:
            // every repetition must reproduce that thread's first results bit for bit
            auto X = load<dtable>(dir + "x.bin", n), Y = load<dtable>(dir + "y.bin", n);
            auto worker = [&](int id, double *res) {
                void *st = nullptr;
                nt2::check(nt2g_stream_create(&st), "stream");
                nt2::options().stream = st;
                dtable x(nt2::of_size(n)), y(nt2::of_size(n));
                x = X * (float)(id + 1);
                y = Y + (float)id;
                res[0] = nt2::sum64(x);
                res[1] = nt2::sum64(x * y);
                res[2] = nt2::sum64(nt2::exp(y) * x);
                int bad = 0;
                for (int k = 0; k < 40; ++k)
                    bad += nt2::sum64(x) != res[0] || nt2::sum64(x * y) != res[1] ||
                           nt2::sum64(nt2::exp(y) * x) != res[2];
                res[3] = bad;
                nt2::check(nt2g_stream_synchronize(st), "stream");
                nt2g_stream_destroy(st);
            };
            double r0[4] = {}, r1[4] = {};
            std::thread t0(worker, 0, r0), t1(worker, 1, r1);
            t0.join();
            t1.join();
            for (const double *r : {r0, r1}) std::printf("%.17g %.17g %.17g %d\n", r[0], r[1], r[2], (int)r[3]);
        } else if (mode == "streams") {
            // one thread, two streams: asynchronous sums in flight on both at once, each stream its own scratch
            auto X = load<dtable>(dir + "x.bin", n), Y = load<dtable>(dir + "y.bin", n);
            void *st[2] = {nullptr, nullptr};
            for (auto &s : st) nt2::check(nt2g_stream_create(&s), "stream");
            nt2::detail::device_buffer res(2 * 16 * sizeof(double));
            double *d = (double *)res.p;
            for (int k = 0; k < 16; ++k)
                for (int s = 0; s < 2; ++s) {
                    nt2::options().stream = st[s];
                    if (s == 0) nt2::sum64_async(X * Y, d + k);
                    else nt2::sum64_async(nt2::exp(X) * Y, d + 16 + k);
                }
            std::vector<double> h(32);
            for (auto s : st) nt2::check(nt2g_stream_synchronize(s), "stream");
            nt2::options().stream = nullptr;
            nt2::check(nt2g_memcpy(h.data(), d, 32 * sizeof(double), 2, nullptr), "results");
            nt2::check(nt2g_stream_synchronize(nullptr), "results");
            for (auto s : st) nt2g_stream_destroy(s);
            for (double v : h) std::printf("%.17g\n", v);
        } else if (mode == "fold") {
            // an M x N table (N = argv[4]): per-column and per-row reductions, then the global forms
            const std::size_t cols = std::strtoull(argv[4], nullptr, 10);
            nt2::table<float> h(nt2::of_size(n, cols));
            auto v = read_bin<float>(dir + "a.bin", n * cols);
            std::memcpy(h.data(), v.data(), v.size() * sizeof(float));
            dtable A;
            A = h;
            save(dir + "sum1.bin", nt2::sum(A, 1));
            save(dir + "sum2.bin", nt2::sum(A, 2));
            save(dir + "max1.bin", nt2::maximum(A, 1));
            save(dir + "min2.bin", nt2::minimum(A, 2));
            save(dir + "mean1.bin", nt2::mean(A, 1));
            save(dir + "norm2_2.bin", nt2::norm2(A, 2));
            save(dir + "hsum1.bin", nt2::sum(h, 1));  // a host table folded in place (or staged)
            save(dir + "cumsum1.bin", nt2::cumsum(A, 1));
            save(dir + "cummax2.bin", nt2::cummax(A, 2));
            save(dir + "var1.bin", nt2::var(A, 0, 1));
            save(dir + "stdev2_w1.bin", nt2::stdev(A, 1, 2));
            save(dir + "meanad1.bin", nt2::meanad(A, 1));
            save(dir + "meanad2.bin", nt2::meanad(A, 2));
            dtable W;
            W = nt2::abs(A);
            save(dir + "wmean1.bin", nt2::wmean(A, W, 1));
            save(dir + "median1.bin", nt2::median(A, 1));
            save(dir + "median2.bin", nt2::median(h, 2));  // a host table, along its rows
            save(dir + "medianad1.bin", nt2::medianad(A));
            save(dir + "asump1.bin", nt2::asump(A, 3.0f, 1));
            save(dir + "normp2.bin", nt2::normp(h, 1.5f, 2));
            std::printf("globalasump %.9g\nglobalnormp %.9g\n", (double)nt2::globalasump(A, 3.0f),
                        (double)nt2::globalnormp(h, 1.5f));
            save(dir + "nanasum2_2.bin", nt2::nanasum2(A, 2));
            save(dir + "trapz1.bin", nt2::trapz(A));
            save(dir + "trapz2.bin", nt2::trapz(h, 2));
            std::printf("globalmeanad %.9g\nglobalnorm_inf %.9g\nglobalnorm_1 %.9g\n", (double)nt2::globalmeanad(A),
                        (double)nt2::globalnorm(h, INFINITY), (double)nt2::globalnorm(A, 1.0f));
            std::printf("globalmedian %.9g\nglobalmedianad %.9g\n", (double)nt2::globalmedian(A),
                        (double)nt2::globalmedianad(h));
            std::int64_t imax = 0, imin = 0;
            const float gmax = nt2::globalmax(A, imax), gmin = nt2::globalmin(h, imin);
            std::printf("globalmax %.9g %lld\nglobalmin %.9g %lld\nglobalmean %.9g\nglobalnorm2 %.9g\n"
                        "globalasum1 %.9g\nglobalvar %.9g\nglobalstdev %.9g\n",
                        (double)gmax, (long long)imax, (double)gmin, (long long)imin, (double)nt2::globalmean(A),
                        (double)nt2::globalnorm2(A), (double)nt2::globalasum1(A), (double)nt2::globalvar(A),
                        (double)nt2::globalstdev(h));
        } else if (mode == "stat") {
            // NT2's distribution functions through the table layer: X on the real line, P in [0, 1]
            auto X = load<dtable>(dir + "x.bin", n), P = load<dtable>(dir + "p.bin", n);
            dtable o(nt2::of_size(n));
            o = nt2::normpdf(X, 0.5f, 1.75f); save(dir + "normpdf3.bin", o);
            o = nt2::norminv(P, 0.5f, 1.75f); save(dir + "norminv3.bin", o);
            o = nt2::expcdf(X, 1.75f); save(dir + "expcdf2.bin", o);
            o = nt2::exppdf(X, 1.75f); save(dir + "exppdf2.bin", o);
            o = nt2::expinv(P, 1.75f); save(dir + "expinv2.bin", o);
            o = nt2::logncdf(X, 0.5f, 1.75f); save(dir + "logncdf3.bin", o);
            o = nt2::lognpdf(X, 0.5f, 1.75f); save(dir + "lognpdf3.bin", o);
            o = nt2::logninv(P, 0.5f, 1.75f); save(dir + "logninv3.bin", o);
            o = nt2::unifcdf(X, -1.25f, 2.5f); save(dir + "unifcdf3.bin", o);
            o = nt2::unifpdf(X); save(dir + "unifpdf.bin", o);
            o = nt2::unifinv(P); save(dir + "unifinv.bin", o);
            o = nt2::caucdf(X, 0.5f, 1.75f); save(dir + "caucdf3.bin", o);
            o = nt2::caupdf(X, 0.5f, 1.75f); save(dir + "caupdf3.bin", o);
            o = nt2::cauinv(P, 0.5f, 1.75f); save(dir + "cauinv3.bin", o);
            o = nt2::cauinv(P, 0.5f); save(dir + "cauinv2.bin", o);
            // boost.simd's selects, minmod, negate, fms and fnma over the same tables
            o = nt2::maxnum(X, P); save(dir + "maxnum.bin", o);
            o = nt2::minnum(P, X); save(dir + "minnum.bin", o);
            o = nt2::maxmag(X, P); save(dir + "maxmag.bin", o);
            o = nt2::minmag(X, P); save(dir + "minmag.bin", o);
            o = nt2::minmod(X, P - 0.5f); save(dir + "minmod.bin", o);
            o = nt2::negate(P, X); save(dir + "negate.bin", o);
            o = nt2::fms(X, P, 0.25f); save(dir + "fms.bin", o);
            o = nt2::fnma(X, P, X); save(dir + "fnma.bin", o);
            o = nt2::divfloor(X, P); save(dir + "divfloor.bin", o);
            o = nt2::divround2even(X, 0.75f); save(dir + "divround2even.bin", o);
            o = nt2::evcdf(X, 0.5f, 1.75f); save(dir + "evcdf3.bin", o);
            o = nt2::evpdf(X, 0.5f, 1.75f); save(dir + "evpdf3.bin", o);
            o = nt2::evinv(P, 0.5f, 1.75f); save(dir + "evinv3.bin", o);
            o = nt2::normpdf(X) + nt2::norminv(P) + nt2::expcdf(X) + nt2::exppdf(X) + nt2::expinv(P) + nt2::logncdf(X) +
                nt2::lognpdf(X) + nt2::logninv(P) + nt2::unifcdf(X) + nt2::caucdf(X) + nt2::caupdf(X) + nt2::evcdf(X) +
                nt2::evpdf(X) + nt2::evinv(P) + nt2::cauinv(P);
            save(dir + "one_param_sum.bin", o);
        } else if (mode == "gen") {
            // generative leaves: NT2's colon (also spelled _), linspace, logspace, alone and in expressions
            using nt2::_;
            dtable c1, c2, c3, l1, l2, g1, g2, w;
            c1 = _(0.f, 9.f);
            c2 = _(0.f, 0.3f, 1.f);
            c3 = nt2::colon(1.f, -0.3f, 0.f);
            l1 = nt2::linspace(-1.f, 1.f, 257);
            l2 = nt2::linspace(0.f, 1.f);
            g1 = nt2::logspace(0.f, 1.f);
            g2 = nt2::logspace(2.f, 3.14159274f, 7);
            w = nt2::sinpi(nt2::linspace(0.f, 2.f, n)) * nt2::colon(1.f, (float)n) + nt2::ones(1, n);
            dtable o1;
            o1 = nt2::zeros(3) + 2.0f;  // a 3 x 3 table of twos
            for (auto *t : {&c1, &c2, &c3, &l1, &l2, &g1, &g2, &w, &o1}) std::printf("%zu\n", t->numel());
            save(dir + "o1.bin", o1);
            save(dir + "c1.bin", c1); save(dir + "c2.bin", c2); save(dir + "c3.bin", c3);
            save(dir + "l1.bin", l1); save(dir + "l2.bin", l2); save(dir + "g1.bin", g1); save(dir + "g2.bin", g2);
            save(dir + "w.bin", w);
        } else if (mode == "sigmadelta") {
            const std::size_t frames = std::strtoull(argv[4], nullptr, 10);
            auto all = read_bin<std::uint8_t>(dir + "frames.bin", n * frames);
            nt2::table<std::uint8_t> hf(nt2::of_size(n));
            std::memcpy(hf.data(), all.data(), n);
            u8table bkg, fr(nt2::of_size(n)), var(nt2::of_size(n)), out(nt2::of_size(n));
            bkg = hf;
            nt2::table<std::uint8_t> ones(nt2::of_size(n));
            std::memset(ones.data(), 1, n);
            var = ones;
            for (std::size_t k = 1; k < frames; ++k) {
                std::memcpy(hf.data(), all.data() + k * n, n);
                fr = hf;
                auto diff = nt2::max(bkg, fr) - nt2::min(bkg, fr);
                auto mul = nt2::adds(nt2::adds(diff, diff), diff);
                nt2::tie(bkg, var, out) =
                    nt2::tie(nt2::selinc(bkg < fr, nt2::seldec(bkg > fr, bkg)),
                             nt2::if_else(diff != std::uint8_t(0), nt2::selinc(var < mul, nt2::seldec(var > mul, var)),
                                          var),
                             nt2::if_zero_else_one(diff < var));
            }
            save(dir + "bkg.bin", bkg);
            save(dir + "var.bin", var);
            save(dir + "label.bin", out);
        } else {
            std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
            return 2;
        }
    } catch (const nt2::gpu_error &e) {
        std::fprintf(stderr, "nt2 gpu error: %s\n", e.what());
        return 1;
    }
    return 0;
}
