// kissfft_gb300::kissfft<scalar_t> -- the reference's C++ facade
// (kissfft.hh:17-189) over the GPU library.
//
// Same interface and meaning as the reference class:
//   kissfft(nfft, inverse)              plan for nfft points, direction fixed
//   assign(nfft, inverse)               re-plan (or flip the direction)
//   transform(in, out[, 0, 1, stride])  nfft-point complex DFT, unscaled
//   transform_real(src, dst)            DFT of 2*nfft reals, packed as the
//                                       reference packs it: dst[0] = (X[0],
//                                       X[nfft]), dst[k] = X[k] for k < nfft;
//                                       with the inverse flag the kernel is
//                                       exp(+i...), i.e. conj(X[k])
// scalar_t is float or double (std::complex<scalar_t> elements).  Buffers
// may be host or device memory; every call returns when its result is in
// place, like the reference's.  Errors throw std::runtime_error with the
// library's message (the reference has no error path).  The stage / fstride
// arguments of transform() are the reference recursion's internals: only
// their defaults are accepted.
//
// Build: -I<repo>/include -I<cuda>/include, link -lkissfft_gb300 -lcudart.
#ifndef KISSFFT_CUDA_HH
#define KISSFFT_CUDA_HH

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>

#include <cuda_runtime_api.h>

#include "kissfft_gb300.h"

namespace kissfft_gb300 {

template <typename scalar_t>
class kissfft {
    static_assert(std::is_same<scalar_t, float>::value || std::is_same<scalar_t, double>::value,
                  "kissfft_gb300::kissfft<scalar_t>: float or double");

   public:
    typedef std::complex<scalar_t> cpx_t;

    kissfft(const std::size_t nfft, const bool inverse) : nfft_(nfft), inverse_(inverse) { plan(); }
    kissfft(const kissfft& o) : nfft_(o.nfft_), inverse_(o.inverse_) { plan(); }
    kissfft(kissfft&& o) noexcept { swap(o); }
    kissfft& operator=(kissfft o) {
        swap(o);
        return *this;
    }
    ~kissfft() { release(); }

    void assign(const std::size_t nfft, const bool inverse) {
        if (nfft == nfft_ && inverse == inverse_) return;
        kissfft tmp(nfft, inverse);
        swap(tmp);
    }

    void transform(const cpx_t* fft_in, cpx_t* fft_out, const std::size_t stage = 0, const std::size_t fstride = 1,
                   const std::size_t in_stride = 1) const {
        if (stage != 0 || fstride != 1)
            throw std::invalid_argument("kissfft::transform: stage and fstride are internal to the recursion");
        if (nfft_ == 0) return;
        const int rc = in_stride == 1 ? kfg_exec(c2c_, fft_in, fft_out, nullptr)
                                      : kfg_exec_stride(c2c_, fft_in, fft_out, (int)in_stride, nullptr);
        check(rc, "transform");
        check(kfg_synchronize(), "transform");
    }

    void transform_real(const scalar_t* const src, cpx_t* const dst) const {
        const std::size_t N = nfft_;
        if (N == 0) return;
        if (!real_) {
            real_ = kfg_plan_real(dtype(), (int)(2 * N), 0);
            if (!real_) fail("transform_real");
            if (cudaMalloc(&d_src_, 2 * N * sizeof(scalar_t)) != cudaSuccess ||
                cudaMalloc(&d_bins_, (N + 1) * sizeof(cpx_t)) != cudaSuccess ||
                cudaMalloc(&d_dst_, N * sizeof(cpx_t)) != cudaSuccess)
                throw std::runtime_error("kissfft::transform_real: device memory");
        }
        cudaStream_t st = (cudaStream_t)kfg_get_stream();
        cuda(cudaMemcpyAsync(d_src_, src, 2 * N * sizeof(scalar_t), cudaMemcpyDefault, st));
        check(kfg_exec(real_, d_src_, d_bins_, nullptr), "transform_real");
        check(kfg_pack_real(dtype(), d_bins_, d_dst_, (long long)N, inverse_ ? 1 : 0, nullptr), "transform_real");
        cuda(cudaMemcpyAsync(dst, d_dst_, N * sizeof(cpx_t), cudaMemcpyDefault, st));
        cuda(cudaStreamSynchronize(st));
    }

    // GPU addition: `batch` transforms of nfft points, packed, in one launch
    void transform_batch(const cpx_t* fft_in, cpx_t* fft_out, long long batch) const {
        check(kfg_exec_batch(c2c_, fft_in, fft_out, batch, 0, 0, nullptr), "transform_batch");
        check(kfg_synchronize(), "transform_batch");
    }

   private:
    static int dtype() { return std::is_same<scalar_t, float>::value ? KFG_FLOAT : KFG_DOUBLE; }
    static void fail(const char* where) {
        throw std::runtime_error(std::string("kissfft::") + where + ": " + kfg_last_error());
    }
    static void check(int rc, const char* where) {
        if (rc != KFG_OK) fail(where);
    }
    static void cuda(cudaError_t e) {
        if (e != cudaSuccess) throw std::runtime_error(std::string("kissfft: ") + cudaGetErrorString(e));
    }
    void plan() {
        if (nfft_ == 0) return;
        c2c_ = kfg_plan_c2c(dtype(), (int)nfft_, inverse_ ? 1 : 0);
        if (!c2c_) fail("kissfft");
    }
    void release() {
        if (c2c_) kfg_plan_free(c2c_);
        if (real_) kfg_plan_free(real_);
        if (d_src_) cudaFree(d_src_);
        if (d_bins_) cudaFree(d_bins_);
        if (d_dst_) cudaFree(d_dst_);
        c2c_ = real_ = nullptr;
        d_src_ = d_bins_ = d_dst_ = nullptr;
    }
    void swap(kissfft& o) noexcept {
        std::swap(nfft_, o.nfft_);
        std::swap(inverse_, o.inverse_);
        std::swap(c2c_, o.c2c_);
        std::swap(real_, o.real_);
        std::swap(d_src_, o.d_src_);
        std::swap(d_bins_, o.d_bins_);
        std::swap(d_dst_, o.d_dst_);
    }

    std::size_t nfft_ = 0;
    bool inverse_ = false;
    kfg_plan* c2c_ = nullptr;
    mutable kfg_plan* real_ = nullptr;  // 2*nfft-point real plan, made on first transform_real
    mutable void* d_src_ = nullptr;
    mutable void* d_bins_ = nullptr;
    mutable void* d_dst_ = nullptr;
};

}  // namespace kissfft_gb300

#endif
