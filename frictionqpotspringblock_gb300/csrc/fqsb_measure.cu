/*
 * Arithmetic throughput of the GPU the library runs on: the denominators of the step kernel's fp64
 * roofline, measured in the same process that times the kernel.
 *
 * The fused step (fqsb_step.cu) is bound by binary64 issue, not by HBM: GB300 retires ~1.6 fp64
 * add / mul / fma per clock per SM, and the step moves part of its binary64 arithmetic onto the
 * integer pipes (fq_soft64.h).  fqsb_measure_arith times independent dependency chains of one
 * operation -- 8 chains per thread, k of them in the integer-pipe form and 8 - k with the fp64
 * instruction -- over 8 CTAs of 256 threads per SM, and reports binary64 operations per second.
 */
#include "fqsb.h"

#include <cuda_runtime.h>

#include "fq_soft64.h"

namespace {

constexpr int CHAINS = 8;

template <int OP, int NSOFT>
__global__ void __launch_bounds__(256) k_arith(double* out, int iters)
{
    int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double x[CHAINS], c[CHAINS];
#pragma unroll
    for (int j = 0; j < CHAINS; ++j) {
        x[j] = __dadd_rn(1.0, __dmul_rn((double)tid, 1e-9)) + (double)j;
        c[j] = OP == 0 ? 1e-3 * (j + 1) : 1.0 + 1e-12 * (j + 1);
    }
    for (int r = 0; r < iters; ++r) {
#pragma unroll
        for (int j = 0; j < CHAINS; ++j) {
            if (OP == 2) {
                x[j] = __fma_rn(x[j], c[j], 1e-9);
            }
            else if (j < NSOFT) {
                x[j] = OP == 0 ? fq_sadd(x[j], c[j]) : fq_smul(x[j], c[j]);
            }
            else {
                x[j] = OP == 0 ? __dadd_rn(x[j], c[j]) : __dmul_rn(x[j], c[j]);
            }
        }
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < CHAINS; ++j) {
        s = __dadd_rn(s, x[j]);
    }
    out[tid] = s;
}

template <int OP, int NSOFT>
cudaError_t launch(double* out, int blocks, int iters, cudaStream_t st)
{
    k_arith<OP, NSOFT><<<blocks, 256, 0, st>>>(out, iters);
    return cudaGetLastError();
}

using Launcher = cudaError_t (*)(double*, int, int, cudaStream_t);

template <int OP>
Launcher pick(int n_soft)
{
    switch (n_soft) {
    case 0: return launch<OP, 0>;
    case 1: return launch<OP, 1>;
    case 2: return launch<OP, 2>;
    case 3: return launch<OP, 3>;
    case 4: return launch<OP, 4>;
    case 5: return launch<OP, 5>;
    case 6: return launch<OP, 6>;
    case 7: return launch<OP, 7>;
    default: return launch<OP, 8>;
    }
}

} // namespace

extern "C" int fqsb_measure_arith(int device, int op, int n_soft, double* gops)
{
    if (!gops || op < 0 || op > 2 || n_soft < 0 || n_soft > CHAINS || (op == 2 && n_soft != 0)) {
        return FQSB_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FQSB_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev || cudaSetDevice(device) != cudaSuccess) {
        return FQSB_ERR_INVALID;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        return FQSB_ERR_CUDA;
    }
    const int blocks = sms * 8;
    /* add / mul in software cost 40-80 instructions: fewer iterations keep a launch near 10 ms */
    const int iters = n_soft > 0 ? 512 : 4096;
    Launcher L = op == 0 ? pick<0>(n_soft) : op == 1 ? pick<1>(n_soft) : pick<2>(0);
    double* out = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = FQSB_ERR_CUDA;
    float ms = 0.0f;
    if (cudaMalloc(&out, sizeof(double) * (size_t)blocks * 256) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        goto done;
    }
    /* first launch warms up (clocks, instruction cache); the second is timed */
    if (L(out, blocks, iters, st) != cudaSuccess || cudaEventRecord(e0, st) != cudaSuccess ||
        L(out, blocks, iters, st) != cudaSuccess || cudaEventRecord(e1, st) != cudaSuccess ||
        cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f) {
        goto done;
    }
    *gops = (double)CHAINS * (double)blocks * 256.0 * (double)iters / ((double)ms * 1e6);
    rc = FQSB_OK;
done:
    if (e0) {
        cudaEventDestroy(e0);
    }
    if (e1) {
        cudaEventDestroy(e1);
    }
    if (st) {
        cudaStreamDestroy(st);
    }
    if (out) {
        cudaFree(out);
    }
    if (rc != FQSB_OK) {
        cudaGetLastError();
    }
    return rc;
}
