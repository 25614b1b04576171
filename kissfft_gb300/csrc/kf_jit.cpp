// Run-time specialisation of the engine kernel with NVRTC.
//
// For one launch step (sample type, mode, plan shape, sub-plan, jobs per
// tile, enumeration) it compiles kf::kf_spec_kernel<...> for sm_103a from
// the engine headers embedded in this library, loads the cubin with
// cudaLibraryLoadData and keeps the kernel handle for the life of the
// process.  Cubins are also kept on disk (KISSFFT_GB300_CACHE, default
// ~/.cache/kissfft_gb300), so a size is compiled once per machine.
//
// Enabled by kfg_set_specialize(1) or KISSFFT_GB300_SPECIALIZE=1; when
// NVRTC fails the caller falls back to the precompiled family kernels.
#include <cuda_runtime.h>
#include <nvrtc.h>
#include <stdio.h>
#include <stdlib.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "kf_plan.h"

namespace kf {

// generated at build time from the device headers (kf_hdrs_gen.cpp)
extern const int kf_hdr_count;
extern const char* const kf_hdr_names[];
extern const char* const kf_hdr_srcs[];

namespace {

std::mutex g_mu;
std::map<std::string, const void*> g_kernels;
std::map<std::string, std::string> g_failed;
std::atomic<int> g_mode{-1};

const char* scalar_name(int dt) {
    switch (dt) {
        case KF_F32: return "float";
        case KF_F64: return "double";
        case KF_Q15: return "short";
        case KF_Q31: return "int";
    }
    return "float";
}

unsigned long long fnv1a(const std::string& s, unsigned long long h = 1469598103934665603ull) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

// Digest of the embedded headers (part of every cache key).  A function
// static initialised once (thread-safe): the autotuner's first compiles run
// on several threads at once.
std::string headers_digest() {
    static const std::string d = [] {
        unsigned long long h = 1469598103934665603ull;
        for (int i = 0; i < kf_hdr_count; ++i) {
            h = fnv1a(kf_hdr_names[i], h);
            h = fnv1a(kf_hdr_srcs[i], h);
        }
        char buf[32];
        snprintf(buf, sizeof(buf), "%016llx", h);
        return std::string(buf);
    }();
    return d;
}

std::string cache_dir() {
    const char* e = getenv("KISSFFT_GB300_CACHE");
    std::string d;
    if (e && *e) {
        d = e;
    } else {
        const char* home = getenv("HOME");
        d = std::string(home && *home ? home : "/tmp") + "/.cache/kissfft_gb300";
    }
    return d;
}

void mkdirs(const std::string& path) {
    std::string cur;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0755);
    }
}

bool read_file(const std::string& p, std::string& out) {
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

void write_file(const std::string& p, const std::string& data) {
    std::string tmp = p + ".tmp" + std::to_string((long long)getpid());
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f) return;
        f.write(data.data(), (std::streamsize)data.size());
    }
    rename(tmp.c_str(), p.c_str());
}

bool compile(const std::string& name, std::string& cubin, std::string& lowered, std::string& err) {
    const char* src = "#include \"kf_spec.cuh\"\n";
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src, "kf_spec_jit.cu", kf_hdr_count, kf_hdr_srcs, kf_hdr_names) != NVRTC_SUCCESS) {
        err = "nvrtcCreateProgram failed";
        return false;
    }
    std::string expr = "&" + name;
    nvrtcAddNameExpression(prog, expr.c_str());
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "--fmad=true"};
    nvrtcResult r = nvrtcCompileProgram(prog, 4, opts);
    if (r != NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        err = std::string("NVRTC: ") + nvrtcGetErrorString(r) + "\n" + log.substr(0, 4000);
        nvrtcDestroyProgram(&prog);
        return false;
    }
    const char* low = nullptr;
    nvrtcGetLoweredName(prog, expr.c_str(), &low);
    lowered = low ? low : "";
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin.resize(n);
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return !lowered.empty() && n > 0;
}

}  // namespace

bool specialize_enabled() {
    int m = g_mode.load();
    if (m < 0) {
        const char* e = getenv("KISSFFT_GB300_SPECIALIZE");
        m = (e && e[0] == '1') ? 1 : 0;
        g_mode.store(m);
    }
    return m == 1;
}

void set_specialize(int on) { g_mode.store(on ? 1 : 0); }

std::string spec_name(const Step& st) {
    std::ostringstream o;
    o << "kf::kf_spec_kernel<" << scalar_name(st.dtype) << "," << st.mode << "," << st.dtype << "," << st.shape_n
      << "," << st.shape_inv << ",0," << st.shape_sub << "," << st.args.J << "," << st.args.col_in << ","
      << st.args.col_out << "," << st.cfg.T << "," << st.cfg.minb << "," << st.args.swz << ">";
    return o.str();
}

// NVRTC compile of a step's specialised kernel without loading it (needs no
// GPU): used by the tests to check the embedded headers.
bool spec_compile_only(const Step& st, std::string& err) {
    std::string cubin, lowered;
    return compile(spec_name(st), cubin, lowered, err);
}

// Kernel handle for a step, compiling (or loading from disk) on first use.
const void* spec_kernel(const Step& st, std::string& err) {
    const std::string name = spec_name(st);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_kernels.find(name);
        if (it != g_kernels.end()) return it->second;
        auto f = g_failed.find(name);
        if (f != g_failed.end()) {
            err = f->second;
            return nullptr;
        }
    }
    // compile outside the lock (NVRTC programs compile concurrently); the
    // first thread to finish registers the kernel
    int ver[2] = {0, 0};
    nvrtcVersion(&ver[0], &ver[1]);
    char key[64];
    snprintf(key, sizeof(key), "%016llx",
             fnv1a(name + "|" + headers_digest() + "|sm_103a|" + std::to_string(ver[0] * 100 + ver[1])));
    const std::string dir = cache_dir();
    const std::string cpath = dir + "/" + key + ".cubin", npath = dir + "/" + key + ".name";
    std::string cubin, lowered;
    if (!(read_file(cpath, cubin) && read_file(npath, lowered))) {
        if (!compile(name, cubin, lowered, err)) {
            std::lock_guard<std::mutex> lk(g_mu);
            g_failed[name] = err;
            return nullptr;
        }
        mkdirs(dir);
        write_file(cpath, cubin);
        write_file(npath, lowered);
    }
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_kernels.find(name);
    if (it != g_kernels.end()) return it->second;
    cudaLibrary_t lib;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        g_failed[name] = err;
        return nullptr;
    }
    cudaKernel_t k;
    e = cudaLibraryGetKernel(&k, lib, lowered.c_str());
    if (e != cudaSuccess) {
        err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e);
        g_failed[name] = err;
        return nullptr;
    }
    e = cudaFuncSetAttribute((const void*)k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) {
        err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
        g_failed[name] = err;
        return nullptr;
    }
    g_kernels[name] = (const void*)k;
    return (const void*)k;
}

}  // namespace kf
