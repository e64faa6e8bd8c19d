/*
 * fqsb_residual_noalloc: the residual reduction without any device allocation.
 *
 * Who needs it: code that must not call cudaMalloc / cudaFree -- for example a host loop running
 * while another thread captures a CUDA graph in global capture mode (where cudaMalloc is a
 * prohibited call), a caller whose device memory is entirely owned by another framework's pool,
 * or a latency-critical loop that cannot afford the implicit device synchronisation of cudaFree.
 * Such a caller passes device arrays it already owns and gets the residual written to a device
 * double it owns; the only scratch (the per-CTA partial sums) lives in a fixed file-scope device
 * array that every GPU loading this library holds until the process exits.
 *
 * Limits and sharing: at most FQSB_NOALLOC_MAX_N entries per call (larger inputs are rejected
 * before any memory is touched).  All calls share the one scratch array and it keeps the previous
 * call's contents; every entry the kernels read is first written by the same call, so nothing has
 * to start at zero.  Calls whose kernels overlap on the GPU (different streams, or different host
 * threads) race on the scratch array and must be serialised by the caller.
 *
 * The first call on each device looks up the scratch array's device address
 * (cudaGetSymbolAddress, with that device current) and caches it; make that first call before any
 * stream capture begins.
 */
#include <mutex>
#include <string>

#include "../../include/fqsb.h"
#include "fqsb_device.cuh"
#include "fqsb_internal.h"

using namespace fqsb;

#define FQSB_NOALLOC_TILE 1024
#define FQSB_NOALLOC_MAX_PARTIALS (FQSB_NOALLOC_MAX_N / FQSB_NOALLOC_TILE)

/* partial sums (sum f^2, sum f_frame^2) of the 1024-entry tiles; 32768 x 16 B = 512 KiB */
static __device__ __align__(256) double2 g_noalloc_scratch[FQSB_NOALLOC_MAX_PARTIALS];

/* tile sums in the fixed pairwise order over the flat index (the order of every residual here) */
__global__ void __launch_bounds__(256) k_noalloc_tiles(const double* f, const double* f_frame, int64_t n,
                                                       double2* partials)
{
    __shared__ double sh[32];
    int64_t lo = (int64_t)blockIdx.x * FQSB_NOALLOC_TILE + threadIdx.x * 4;
    double x[4], y[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        x[j] = 0.0;
        y[j] = 0.0;
        if (lo + j < n) {
            double a = f[lo + j], b = f_frame[lo + j];
            x[j] = FQ_MUL(a, a);
            y[j] = FQ_MUL(b, b);
        }
    }
    double rx = FQ_ADD(FQ_ADD(x[0], x[1]), FQ_ADD(x[2], x[3]));
    double ry = FQ_ADD(FQ_ADD(y[0], y[1]), FQ_ADD(y[2], y[3]));
    double sx = cta_tree(rx, sh);
    __syncthreads();
    double sy = cta_tree(ry, sh);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = make_double2(sx, sy);
    }
}

/* tree over the tile sums, then residual = |f| / |f_frame| (or |f| when |f_frame| == 0), detail.h:1512-1520 */
__global__ void __launch_bounds__(256) k_noalloc_final(const double2* partials, int64_t G, double* out)
{
    __shared__ double sh[32];
    int64_t P = next_pow2(G);
    int T = blockDim.x;
    double x = 0.0, y = 0.0;
    if (P <= T) {
        if (threadIdx.x < G) {
            x = partials[threadIdx.x].x;
            y = partials[threadIdx.x].y;
        }
    }
    else {
        int64_t per = P / T, lo = (int64_t)threadIdx.x * per;
        x = serial_tree([&](int64_t i) { return i < G ? partials[i].x : 0.0; }, lo, per);
        y = serial_tree([&](int64_t i) { return i < G ? partials[i].y : 0.0; }, lo, per);
    }
    double sx = cta_tree(x, sh);
    __syncthreads();
    double sy = cta_tree(y, sh);
    if (threadIdx.x == 0) {
        double r_fres = FQ_SQRT(sx), r_fext = FQ_SQRT(sy);
        *out = r_fext != 0.0 ? FQ_DIV(r_fres, r_fext) : r_fres;
    }
}

/* device address of g_noalloc_scratch, looked up once per device with that device current */
static std::mutex g_noalloc_mutex;
static void* g_noalloc_addr[256];

static int noalloc_scratch(int device, void** ptr)
{
    if (device < 0 || device >= 256) {
        return FQSB_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_global_error(std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") +
                             cudaGetErrorString(e));
            return FQSB_ERR_CUDA;
        }
        g_noalloc_addr[device] = p;
    }
    *ptr = g_noalloc_addr[device];
    return FQSB_OK;
}

extern "C" int fqsb_residual_noalloc(const double* f_device, const double* f_frame_device, int64_t n,
                                     double* residual_device, void* stream)
{
    if (!f_device || !f_frame_device || !residual_device) {
        set_global_error("fqsb_residual_noalloc: null pointer");
        return FQSB_ERR_INVALID;
    }
    if (n < 1 || n > FQSB_NOALLOC_MAX_N) {
        set_global_error("fqsb_residual_noalloc: n must be in [1, " + std::to_string((long long)FQSB_NOALLOC_MAX_N) +
                         "], got " + std::to_string((long long)n));
        return FQSB_ERR_INVALID;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) {
        set_global_error(std::string("fqsb_residual_noalloc: ") + cudaGetErrorString(e));
        return FQSB_ERR_CUDA;
    }
    void* scratch = nullptr;
    int rc = noalloc_scratch(device, &scratch);
    if (rc) {
        return rc;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int64_t G = (n + FQSB_NOALLOC_TILE - 1) / FQSB_NOALLOC_TILE;
    k_noalloc_tiles<<<(unsigned)G, 256, 0, st>>>(f_device, f_frame_device, n, (double2*)scratch);
    k_noalloc_final<<<1, 256, 0, st>>>((const double2*)scratch, G, residual_device);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error(std::string("fqsb_residual_noalloc: ") + cudaGetErrorString(e));
        return FQSB_ERR_CUDA;
    }
    return FQSB_OK;
}
