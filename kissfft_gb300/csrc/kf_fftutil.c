/*
 * fftutil for the GPU library: the stream front end of the reference's
 * tools/fftutil.c (options, frame sizes and byte layout of
 * tools/fftutil.c:19-126), so raw-binary pipelines and scripts written for
 * it drive the GPU transforms unchanged.
 *
 *   fftutil_cuda-<type> [-n d1[,d2,...]] [-i] [-R] [infile|-] [outfile|-]
 *
 *   -n  transform size, or the dimensions of an N-D transform (default 1024)
 *   -i  inverse
 *   -R  real samples (kiss_fftr / kiss_fftndr); the inverse reads bins
 *
 * Input is read as whole frames of the build's sample type (interleaved
 * complex, or reals with -R); a trailing partial frame is ignored, as in
 * the reference.  Unlike the reference, which transforms one frame per
 * call, frames are read in chunks of up to 64 MiB into page-locked memory
 * and each chunk is one batched call that the GPU reads and writes in place
 * (kfg_exec_batch on pinned host buffers).
 *
 * Built once per sample type: -DKF_TOOL_DTYPE=0 float, 1 double,
 * 2 int16_t (Q15), 3 int32_t (Q31).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <cuda_runtime_api.h>

#include "kissfft_gb300.h"

#ifndef KF_TOOL_DTYPE
#define KF_TOOL_DTYPE 0
#endif

static const size_t kScalar[4] = {4, 8, 2, 4};
static const size_t kChunkBytes = (size_t)64 << 20;

static int parse_dims(char* arg, int* dims, int maxd) {
    int nd = 0;
    char* p = arg;
    while (p && nd < maxd) {
        char* c = strchr(p, ',');
        if (c) *c++ = '\0';
        dims[nd++] = atoi(p);
        p = c;
    }
    return nd;
}

static void usage(void) {
    fprintf(stderr,
            "usage options:\n"
            "\t-n d1[,d2,d3...]: fft dimension(s)\n"
            "\t-i : inverse\n"
            "\t-R : real input samples, not complex\n");
    exit(1);
}

int main(int argc, char** argv) {
    int inverse = 0, real = 0, ndims = 1, dims[32] = {1024};
    int c;
    while ((c = getopt(argc, argv, "n:iR")) != -1) {
        switch (c) {
            case 'n': ndims = parse_dims(optarg, dims, 32); break;
            case 'i': inverse = 1; break;
            case 'R': real = 1; break;
            default: usage();
        }
    }
    FILE* fin = stdin;
    FILE* fout = stdout;
    if (optind < argc) {
        if (strcmp(argv[optind], "-") != 0 && !(fin = fopen(argv[optind], "rb"))) {
            perror(argv[optind]);
            return 1;
        }
        ++optind;
    }
    if (optind < argc) {
        if (strcmp(argv[optind], "-") != 0 && !(fout = fopen(argv[optind], "wb"))) {
            perror(argv[optind]);
            return 1;
        }
        ++optind;
    }
    const int dt = KF_TOOL_DTYPE;
    const size_t sc = kScalar[dt];
    long long prod = 1;
    for (int i = 0; i < ndims; ++i) {
        if (dims[i] < 1) usage();
        prod *= dims[i];
    }
    kfg_plan* p;
    size_t in_frame, out_frame; /* bytes */
    if (!real) {
        p = ndims == 1 ? kfg_plan_c2c(dt, dims[0], inverse) : kfg_plan_nd(dt, dims, ndims, inverse);
        in_frame = out_frame = (size_t)prod * 2 * sc;
    } else {
        const long long last = dims[ndims - 1];
        const long long bins = prod / last * (last / 2 + 1);
        p = ndims == 1 ? kfg_plan_real(dt, dims[0], inverse) : kfg_plan_ndr(dt, dims, ndims, inverse);
        in_frame = inverse ? (size_t)bins * 2 * sc : (size_t)prod * sc;
        out_frame = inverse ? (size_t)prod * sc : (size_t)bins * 2 * sc;
    }
    if (!p) {
        fprintf(stderr, "[ERROR] fftutil: %s\n", kfg_last_error());
        return 1;
    }
    size_t frames = kChunkBytes / (in_frame > out_frame ? in_frame : out_frame);
    if (frames < 1) frames = 1;
    unsigned char *ib = NULL, *ob = NULL;
    if (cudaHostAlloc((void**)&ib, frames * in_frame, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&ob, frames * out_frame, cudaHostAllocDefault) != cudaSuccess) {
        fprintf(stderr, "[ERROR] fftutil: no page-locked host memory\n");
        return 1;
    }
    int rc = 0;
    for (;;) {
        const size_t got = fread(ib, in_frame, frames, fin); /* whole frames only */
        if (got == 0) break;
        if (kfg_exec_batch(p, ib, ob, (long long)got, 0, 0, NULL) != KFG_OK) {
            fprintf(stderr, "[ERROR] fftutil: %s\n", kfg_last_error());
            rc = 1;
            break;
        }
        if (fwrite(ob, out_frame, got, fout) != got) {
            perror("fftutil: write");
            rc = 1;
            break;
        }
        if (got < frames) break;
    }
    cudaFreeHost(ib);
    cudaFreeHost(ob);
    kfg_plan_free(p);
    if (fout != stdout) fclose(fout);
    if (fin != stdin) fclose(fin);
    return rc;
}
