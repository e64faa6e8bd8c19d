// Device check of the integer-pipe binary64 add / sub / mul (fq_soft64.h) against the GPU's own
// fp64 instructions on pseudo-random operands (raw bit patterns, close exponents, near cancellation,
// few-bit significands).  Usage: soft64_device_check <blocks> <cases per thread>.  Prints the number
// of mismatching triples and up to 8 of them; exits 1 on any mismatch or CUDA error.
#include <cstdio>
#include <cstdlib>
#include "fq_soft64.h"

__device__ uint64_t next64(uint64_t& s)
{
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__device__ bool same(double x, double y)
{
    return (x != x && y != y) || __double_as_longlong(x) == __double_as_longlong(y);
}

__global__ void k_check(unsigned long long* bad, unsigned long long* first, int per)
{
    uint64_t s = (0x1234567ULL + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * 0x2545F4914F6CDD1DULL;
    for (int i = 0; i < per; ++i) {
        uint64_t A = next64(s), B = next64(s);
        int fam = i & 3;
        if (fam == 1) {
            B = (B & 0x800fffffffffffffULL) | ((((A >> 52) & 0x7ff) + (next64(s) % 9) - 4) & 0x7ff) << 52;
        }
        else if (fam == 2) {
            B = (A ^ 0x8000000000000000ULL) ^ (next64(s) & ((1ULL << (next64(s) % 53)) - 1));
        }
        else if (fam == 3) {
            B = B & ~((1ULL << (next64(s) % 52)) - 1);
            A = A & ~((1ULL << (next64(s) % 52)) - 1);
        }
        double a = __longlong_as_double((long long)A), b = __longlong_as_double((long long)B);
        int m = (same(fq_sadd(a, b), __dadd_rn(a, b)) ? 0 : 1) | (same(fq_ssub(a, b), __dsub_rn(a, b)) ? 0 : 2) |
                (same(fq_smul(a, b), __dmul_rn(a, b)) ? 0 : 4);
        if (m) {
            unsigned long long k = atomicAdd(bad, 1ULL);
            if (k < 8) {
                first[3 * k] = A;
                first[3 * k + 1] = B;
                first[3 * k + 2] = (unsigned long long)m;
            }
        }
    }
}

int main(int argc, char** argv)
{
    int blocks = argc > 1 ? atoi(argv[1]) : 608;
    int per = argc > 2 ? atoi(argv[2]) : 1024;
    unsigned long long *bad = nullptr, *first = nullptr;
    if (cudaMalloc(&bad, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&first, 24 * sizeof(unsigned long long)) != cudaSuccess) {
        printf("cuda alloc failed\n");
        return 1;
    }
    cudaMemset(bad, 0, sizeof(unsigned long long));
    k_check<<<blocks, 256>>>(bad, first, per);
    unsigned long long hb = 0, hf[24] = {0};
    cudaMemcpy(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
    cudaMemcpy(hf, first, sizeof(hf), cudaMemcpyDeviceToHost);
    cudaError_t e = cudaDeviceSynchronize();
    printf("cases %llu mismatches %llu status %s\n", (unsigned long long)blocks * 256ULL * (unsigned long long)per, hb,
           cudaGetErrorString(e));
    for (unsigned long long k = 0; k < hb && k < 8; ++k) {
        printf("A=%016llx B=%016llx ops=%llu\n", hf[3 * k], hf[3 * k + 1], hf[3 * k + 2]);
    }
    cudaFree(bad);
    cudaFree(first);
    return (e != cudaSuccess || hb != 0) ? 1 : 0;
}
