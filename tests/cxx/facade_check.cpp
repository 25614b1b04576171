// Checks kissfft_gb300::kissfft<T> (include/kissfft_cuda.hh) against a
// direct O(N^2) DFT in long double, the way a reference kissfft.hh user
// would call it: host and device buffers, inverse flag, strided input,
// assign(), transform_real() packing.  Prints one line per check with its
// relative L2 error and exits non-zero if any check is beyond its bound
// (float 2e-7*log2(N), double 1e-15*log2(N), times 4 for transform_real).
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

#include "kissfft_cuda.hh"

typedef long double LD;

static unsigned long long g_seed = 7;
static double urand() {
    g_seed = g_seed * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(g_seed >> 11) / 9007199254740992.0 * 2.0 - 1.0;
}

template <typename T>
static std::vector<std::complex<LD>> dft(const std::vector<std::complex<T>>& x, size_t stride, size_t n, bool inv) {
    std::vector<std::complex<LD>> y(n);
    const LD s = (inv ? 2 : -2) * acosl(-1.0L) / (LD)n;
    for (size_t k = 0; k < n; ++k) {
        std::complex<LD> acc = 0;
        for (size_t j = 0; j < n; ++j) {
            const LD ph = s * (LD)((k * j) % n);
            acc += std::complex<LD>(x[j * stride].real(), x[j * stride].imag()) * std::complex<LD>(cosl(ph), sinl(ph));
        }
        y[k] = acc;
    }
    return y;
}

template <typename T>
static double relerr(const std::complex<T>* got, const std::vector<std::complex<LD>>& ref) {
    LD e = 0, r = 0;
    for (size_t k = 0; k < ref.size(); ++k) {
        const std::complex<LD> g(got[k].real(), got[k].imag());
        e += std::norm(g - ref[k]);
        r += std::norm(ref[k]);
    }
    return (double)sqrtl(e / (r > 0 ? r : 1));
}

static int bad = 0;
static void report(const char* what, size_t n, double err, double bound) {
    const bool ok = err <= bound;
    printf("%-28s n=%-6zu relerr=%.3e bound=%.3e %s\n", what, n, err, bound, ok ? "OK" : "FAIL");
    if (!ok) bad = 1;
}

template <typename T>
static void check_type(double unit) {
    typedef std::complex<T> C;
    for (size_t n : {480, 1000, 1024, 17}) {
        const double bound = unit * std::max(1.0, std::log2((double)n));
        std::vector<C> x(3 * n), y(n);
        for (auto& v : x) v = C((T)urand(), (T)urand());
        for (bool inv : {false, true}) {
            kissfft_gb300::kissfft<T> f(n, inv);
            f.transform(x.data(), y.data());
            report(inv ? "transform inverse (host)" : "transform forward (host)", n, relerr(y.data(), dft(x, 1, n, inv)),
                   bound);
            f.transform(x.data(), y.data(), 0, 1, 3);
            report("transform in_stride 3", n, relerr(y.data(), dft(x, 3, n, inv)), bound);
        }
        // device buffers, and assign() flipping the direction
        kissfft_gb300::kissfft<T> f(n, false);
        f.assign(n, true);
        C *dx = nullptr, *dy = nullptr;
        cudaMalloc((void**)&dx, n * sizeof(C));
        cudaMalloc((void**)&dy, n * sizeof(C));
        cudaMemcpy(dx, x.data(), n * sizeof(C), cudaMemcpyHostToDevice);
        f.transform(dx, dy);
        cudaMemcpy(y.data(), dy, n * sizeof(C), cudaMemcpyDeviceToHost);
        report("transform inverse (device)", n, relerr(y.data(), dft(x, 1, n, true)), bound);
        cudaFree(dx);
        cudaFree(dy);
    }
    for (size_t N : {256, 500}) {  // transform_real: 2N reals
        const double bound = 4 * unit * std::log2(2.0 * N);
        std::vector<T> src(2 * N);
        for (auto& v : src) v = (T)urand();
        std::vector<std::complex<T>> sx(2 * N);
        for (size_t i = 0; i < 2 * N; ++i) sx[i] = std::complex<T>(src[i], 0);
        for (bool inv : {false, true}) {
            kissfft_gb300::kissfft<T> f(N, inv);
            std::vector<C> dst(N);
            f.transform_real(src.data(), dst.data());
            auto X = dft(sx, 1, 2 * N, inv);
            std::vector<std::complex<LD>> ref(N);
            ref[0] = std::complex<LD>(X[0].real(), X[N].real());  // the reference's packing
            for (size_t k = 1; k < N; ++k) ref[k] = X[k];
            report(inv ? "transform_real inverse" : "transform_real forward", 2 * N, relerr(dst.data(), ref), bound);
        }
    }
    // batched addition
    {
        const size_t n = 1024, b = 8;
        std::vector<C> x(n * b), y(n * b);
        for (auto& v : x) v = C((T)urand(), (T)urand());
        kissfft_gb300::kissfft<T> f(n, false);
        f.transform_batch(x.data(), y.data(), (long long)b);
        double worst = 0;
        for (size_t k = 0; k < b; ++k) {
            std::vector<C> row(x.begin() + k * n, x.begin() + (k + 1) * n);
            worst = std::max(worst, relerr(y.data() + k * n, dft(row, 1, n, false)));
        }
        report("transform_batch", n, worst, unit * 10);
    }
}

int main() {
    check_type<float>(2e-7);
    check_type<double>(1e-15);
    printf("%s\n", bad ? "FAILED" : "ALL OK");
    return bad;
}
