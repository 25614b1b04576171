"""Builds the GPU libraries in-tree (no cmake, no pip install).

    python -m kissfft_gb300.build

produces, under kissfft_gb300/lib/:
    libkissfft_gb300.so          core: plans, schedules, sm_103a kernels
    libkissfft_cuda-<type>.so    drop-in C ABI (include/kiss_fft_cuda.h) for
                                 type in float, double, int16_t, int32_t
    fftutil_cuda-<type>          the tools/fftutil.c stream front end on the GPU

The kernels are compiled once per (sample type, kernel family, transform
mode) part from csrc/kf_inst.cu, all translation units in parallel, for
sm_103a only.
Objects are cached by a hash of their sources and flags.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-I", CSRC, "-I", INC] + ARCH
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas", "-I", CSRC, "-I", INC,
            "-I", os.path.join(CUDA_HOME, "include")]
DTYPES = ["float", "double", "int16_t", "int32_t"]
DROPIN_DEFS = {
    "float": ["-DKF_DROPIN_DTYPE=0", "-Dkiss_fft_scalar=float"],
    "double": ["-DKF_DROPIN_DTYPE=1", "-Dkiss_fft_scalar=double"],
    "int16_t": ["-DKF_DROPIN_DTYPE=2", "-DFIXED_POINT=16"],
    "int32_t": ["-DKF_DROPIN_DTYPE=3", "-DFIXED_POINT=32"],
}
HEADERS = ["kf_arith.cuh", "kf_desc.h", "kf_engine.cuh", "kf_runner.cuh", "kf_kernels.cuh", "kf_plan.h",
           "kf_shape.h", "kf_stdint.h", "kf_device.cuh", "kf_spec.cuh"]
# the device headers NVRTC compiles specialised kernels from (embedded in the core library)
JIT_HEADERS = ["kf_spec.cuh", "kf_device.cuh", "kf_runner.cuh", "kf_engine.cuh", "kf_arith.cuh", "kf_desc.h",
               "kf_shape.h", "kf_stdint.h"]


def _gen_headers_cpp(out):
    parts = ["// generated by kissfft_gb300/build.py: device headers for NVRTC", "namespace kf {",
             "extern const int kf_hdr_count = %d;" % len(JIT_HEADERS),
             "extern const char* const kf_hdr_names[] = {%s};" % ", ".join('"%s"' % h for h in JIT_HEADERS),
             "extern const char* const kf_hdr_srcs[] = {"]
    for h in JIT_HEADERS:
        with open(os.path.join(CSRC, h)) as f:
            txt = f.read()
        chunks = [txt[i:i + 12000] for i in range(0, len(txt), 12000)]
        parts.append("    " + " ".join('R"KFHDR(%s)KFHDR"' % c for c in chunks) + ",")
    parts += ["};", "}  // namespace kf", ""]
    data = "\n".join(parts)
    if not (os.path.exists(out) and open(out).read() == data):
        with open(out, "w") as f:
            f.write(data)


def core_lib():
    return os.path.join(LIB, "libkissfft_gb300.so")


def dropin_lib(dtype):
    return os.path.join(LIB, "libkissfft_cuda-%s.so" % dtype)


def fftutil_bin(dtype):
    """The raw-binary stream tool of one sample type (csrc/kf_fftutil.c)."""
    return os.path.join(LIB, "fftutil_cuda-%s" % dtype)


# (sample type, kernel family, transform mode) parts of csrc/kf_inst.cu: one
# translation unit each, so the build runs them in parallel.  Modes 0..2 are
# c2c, r2c, c2r; mode 3, the fused fast FIR, exists for float families 0 and 1.
INST_PARTS = [(dt, fam, mode) for dt in range(4) for fam in range(3) for mode in range(4)
              if mode < 3 or (dt == 0 and fam < 2)]


def _cost(task):
    """Rough compile-time rank of a task (bigger first)."""
    name = os.path.basename(task[2])
    if name.startswith("kf_inst_"):
        dt, fam, _ = (int(x) for x in name[len("kf_inst_"):-2].split("_"))
        return (3 if dt == 0 else 1) * (1 + fam)
    return 0


def _digest(paths, flags):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(repr(flags).encode())
    return h.hexdigest()[:16]


def _hdrs():
    return [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INC, "kissfft_gb300.h"),
                                                        os.path.join(INC, "kiss_fft_cuda.h")]


def _compile(cmd, src_paths, out, verbose):
    stamp = out + ".hash"
    dg = _digest(src_paths, cmd)
    if os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == dg:
        return out
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    with open(stamp, "w") as f:
        f.write(dg)
    return out


def build(verbose=False, jobs=None):
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s" % NVCC)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    hdrs = _hdrs()
    tasks = []
    for dt, fam, mode in INST_PARTS:
        out = os.path.join(BUILD, "kf_inst_%d_%d_%d.o" % (dt, fam, mode))
        cmd = [NVCC] + NVFLAGS + ["-DKF_INST_DT=%d" % dt, "-DKF_INST_FAM=%d" % fam, "-DKF_INST_MODE=%d" % mode,
                                  "-c", os.path.join(CSRC, "kf_inst.cu"), "-o", out]
        tasks.append((cmd, [os.path.join(CSRC, "kf_inst.cu")] + hdrs, out))
    out = os.path.join(BUILD, "kf_lib.o")
    tasks.append(([NVCC] + NVFLAGS + ["-c", os.path.join(CSRC, "kf_lib.cu"), "-o", out],
                  [os.path.join(CSRC, "kf_lib.cu")] + hdrs, out))
    out = os.path.join(BUILD, "kf_serve.o")
    tasks.append(([NVCC] + NVFLAGS + ["-c", os.path.join(CSRC, "kf_serve.cu"), "-o", out],
                  [os.path.join(CSRC, "kf_serve.cu")] + hdrs, out))
    out = os.path.join(BUILD, "kf_noalloc.o")
    tasks.append(([NVCC] + NVFLAGS + ["-c", os.path.join(CSRC, "kf_noalloc.cu"), "-o", out],
                  [os.path.join(CSRC, "kf_noalloc.cu")] + hdrs, out))
    out = os.path.join(BUILD, "kf_plan.o")
    tasks.append((["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, "kf_plan.cpp"), "-o", out],
                  [os.path.join(CSRC, "kf_plan.cpp")] + hdrs, out))
    out = os.path.join(BUILD, "kf_jit.o")
    tasks.append((["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, "kf_jit.cpp"), "-o", out],
                  [os.path.join(CSRC, "kf_jit.cpp")] + hdrs, out))
    gen = os.path.join(BUILD, "kf_hdrs_gen.cpp")
    _gen_headers_cpp(gen)
    out = os.path.join(BUILD, "kf_hdrs_gen.o")
    tasks.append((["g++"] + CXXFLAGS + ["-c", gen, "-o", out], [gen], out))
    jobs = jobs or max(1, os.cpu_count() or 1)
    # longest first: float (three-stage register groups), then the general and smooth families
    tasks.sort(key=_cost, reverse=True)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda t: _compile(t[0], t[1], t[2], verbose), tasks))
    core = core_lib()
    link = [NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", core] + objs + ["-lnvrtc"]
    _compile(link, objs, core, verbose)
    for dt in DTYPES:
        out = dropin_lib(dt)
        cmd = ["g++"] + CXXFLAGS + DROPIN_DEFS[dt] + ["-shared", "-o", out, os.path.join(CSRC, "kf_dropin.cpp"),
                                                      "-L", LIB, "-lkissfft_gb300",
                                                      "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart",
                                                      "-Wl,-rpath,$ORIGIN"]
        _compile(cmd, [os.path.join(CSRC, "kf_dropin.cpp"), core] + hdrs, out, verbose)
    for i, dt in enumerate(DTYPES):
        out = fftutil_bin(dt)
        cmd = ["gcc", "-O2", "-Wall", "-DKF_TOOL_DTYPE=%d" % i, "-I", INC, "-I", os.path.join(CUDA_HOME, "include"),
               os.path.join(CSRC, "kf_fftutil.c"), "-o", out, "-L", LIB, "-lkissfft_gb300",
               "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN"]
        _compile(cmd, [os.path.join(CSRC, "kf_fftutil.c"), core] + hdrs, out, verbose)
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIB)
