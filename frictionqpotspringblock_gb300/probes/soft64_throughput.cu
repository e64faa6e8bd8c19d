// Throughput of the integer-pipe binary64 add / mul (csrc/fq_soft64.h) against the fp64 pipe, alone
// and mixed (k of 8 independent chains per thread in software), plus a device exactness check of
// add / sub / mul against the GPU's own instructions.  Build and run from the repository root:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -fmad=false \
//        -Ifrictionqpotspringblock_gb300/csrc frictionqpotspringblock_gb300/probes/soft64_throughput.cu \
//        -o soft64_throughput && ./soft64_throughput
#include <cstdio>
#include <cstdint>
#include "fq_soft64.h"

#define CH 8
template <int NSOFT, int OP>  // OP 0 add, 1 mul
__global__ void __launch_bounds__(256) k_thr(double* out, int R)
{
    int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double x[CH], c[CH];
#pragma unroll
    for (int j = 0; j < CH; ++j) {
        x[j] = 1.0 + (double)tid * 1e-9 + j;
        c[j] = OP == 0 ? 1e-3 * (j + 1) : 1.0 + 1e-12 * (j + 1);
    }
    for (int r = 0; r < R; ++r) {
#pragma unroll
        for (int j = 0; j < CH; ++j) {
            if (j < NSOFT) {
                x[j] = OP == 0 ? fq_sadd(x[j], c[j]) : fq_smul(x[j], c[j]);
            } else {
                x[j] = OP == 0 ? __dadd_rn(x[j], c[j]) : __dmul_rn(x[j], c[j]);
            }
        }
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < CH; ++j) s = __dadd_rn(s, x[j]);
    out[tid] = s;
}

__device__ uint64_t sm64(uint64_t& s)
{
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__global__ void k_check(unsigned long long* bad, unsigned long long* first, int per)
{
    uint64_t s = 0x1234567ULL + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    s *= 0x2545F4914F6CDD1DULL;
    for (int i = 0; i < per; ++i) {
        uint64_t A = sm64(s), B = sm64(s);
        int fam = i & 3;
        if (fam == 1) { // close exponents
            B = (B & 0x800fffffffffffffULL) | ((((A >> 52) & 0x7ff) + (sm64(s) % 9) - 4) & 0x7ff) << 52;
        } else if (fam == 2) { // cancellation
            B = (A ^ 0x8000000000000000ULL) ^ (sm64(s) & ((1ULL << (sm64(s) % 53)) - 1));
        } else if (fam == 3) { // few-bit
            B = B & ~((1ULL << (sm64(s) % 52)) - 1);
            A = A & ~((1ULL << (sm64(s) % 52)) - 1);
        }
        double a = __longlong_as_double((long long)A), b = __longlong_as_double((long long)B);
        double r1 = fq_sadd(a, b), h1 = __dadd_rn(a, b);
        double r2 = fq_ssub(a, b), h2 = __dsub_rn(a, b);
        double r3 = fq_smul(a, b), h3 = __dmul_rn(a, b);
        bool ok1 = (r1 != r1 && h1 != h1) || __double_as_longlong(r1) == __double_as_longlong(h1);
        bool ok2 = (r2 != r2 && h2 != h2) || __double_as_longlong(r2) == __double_as_longlong(h2);
        bool ok3 = (r3 != r3 && h3 != h3) || __double_as_longlong(r3) == __double_as_longlong(h3);
        if (!(ok1 && ok2 && ok3)) {
            unsigned long long k = atomicAdd(bad, 1ULL);
            if (k < 8) { first[3 * k] = A; first[3 * k + 1] = B; first[3 * k + 2] = (ok1 ? 0 : 1) | (ok2 ? 0 : 2) | (ok3 ? 0 : 4); }
        }
    }
}

template <int NS, int OP>
float run(double* out, int blocks, int R)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    k_thr<NS, OP><<<blocks, 256>>>(out, R);
    cudaEventRecord(e0);
    k_thr<NS, OP><<<blocks, 256>>>(out, R);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)blocks * 256 * R * CH;
    printf("OP=%s soft=%d/8: %.3f ms  %.1f Gop/s\n", OP ? "mul" : "add", NS, ms, ops / ms / 1e6);
    return ms;
}

int main()
{
    int blocks = 152 * 8, R = 512;
    double* out; cudaMalloc(&out, sizeof(double) * blocks * 256);
    run<0,0>(out, blocks, R); run<2,0>(out, blocks, R); run<4,0>(out, blocks, R); run<6,0>(out, blocks, R); run<8,0>(out, blocks, R);
    run<0,1>(out, blocks, R); run<2,1>(out, blocks, R); run<4,1>(out, blocks, R); run<6,1>(out, blocks, R); run<8,1>(out, blocks, R);
    unsigned long long *bad, *first; cudaMalloc(&bad, 8); cudaMalloc(&first, 8 * 24); cudaMemset(bad, 0, 8);
    k_check<<<152 * 4, 256>>>(bad, first, 4096);
    unsigned long long hb, hf[24]; cudaMemcpy(&hb, bad, 8, cudaMemcpyDeviceToHost); cudaMemcpy(hf, first, 8 * 24, cudaMemcpyDeviceToHost);
    printf("device check: %llu mismatches in %llu triples\n", hb, (unsigned long long)152 * 4 * 256 * 4096);
    for (unsigned long long k = 0; k < hb && k < 8; ++k) printf("  A=%016llx B=%016llx ops=%llu\n", hf[3*k], hf[3*k+1], hf[3*k+2]);
    cudaError_t e = cudaDeviceSynchronize();
    printf("status %s\n", cudaGetErrorString(e));
    return e != cudaSuccess;
}
