// Bit-for-bit check of quotient() (luma_gb300/csrc/quotient.cuh) against
// CUDA's FP64 division: pseudo-random operands over several exponent spans
// plus special values (signed zeros, subnormals, infinities, NaN, operands
// at the fallback bounds).  Prints the mismatch count; exit status 1 on any.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "quotient.cuh"

using luma::quotient;

__device__ __forceinline__ uint64_t mix(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
    return x;
}
__device__ double draw(uint64_t s, int span) {
    const uint64_t m = mix(s);
    const uint64_t mant = m & 0xfffffffffffffull;
    const int e = 1023 + (int)((m >> 52) % (uint64_t)(2 * span + 1)) - span;
    const uint64_t sign = (mix(s ^ 0x9e3779b97f4a7c15ull) & 1ull) << 63;
    return __longlong_as_double((long long)(sign | ((uint64_t)e << 52) | mant));
}
__device__ bool same(double x, double y) {
    if (x != x && y != y) return true;  // NaN against NaN
    return __double_as_longlong(x) == __double_as_longlong(y);
}
__global__ void check_random(unsigned long long *bad, unsigned long long base, int per, int span) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long nb = 0;
    for (int k = 0; k < per; ++k) {
        const uint64_t s = base + (t * per + k) * 2;
        const double a = draw(s, span), b = draw(s + 1, span);
        if (!same(quotient(a, b, 1.0 / b), a / b)) ++nb;
    }
    if (nb) atomicAdd(bad, nb);
}
__global__ void check_special(unsigned long long *bad, const double *v, int nv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv * nv) return;
    const double a = v[i / nv], b = v[i % nv];
    if (!same(quotient(a, b, 1.0 / b), a / b)) atomicAdd(bad, 1ull);
}
int main() {
    unsigned long long *bad = nullptr, hbad = 0, total = 0;
    if (cudaMalloc(&bad, sizeof hbad) != cudaSuccess) return 2;
    cudaMemset(bad, 0, sizeof hbad);
    const int blocks = 152 * 8, threads = 256, per = 64;
    for (int span : {2, 40, 399, 420}) {
        for (int rep = 0; rep < 4; ++rep) {
            check_random<<<blocks, threads>>>(bad, (unsigned long long)rep * blocks * threads * per * 2 + span * 7919ull,
                                              per, span);
            total += (unsigned long long)blocks * threads * per;
        }
    }
    const double inf = __builtin_inf(), nan = __builtin_nan("");
    const double sv[] = {0.0, -0.0, 1.0, -1.0, 3.0, 1.0 / 3.0, 0.1, 7.0e-3, 2.2250738585072014e-308, 4.9e-324,
                         -4.9e-324, 1.7976931348623157e308, inf, -inf, nan, 0x1p400, 0x1p401, 0x1p-400, 0x1p-401,
                         0x1.fffffffffffffp399, 0x1.0000000000001p-400, 6.0, 1.9999999999999998, 0.9999999999999999};
    const int nv = sizeof(sv) / sizeof(sv[0]);
    double *dv = nullptr;
    cudaMalloc(&dv, sizeof sv);
    cudaMemcpy(dv, sv, sizeof sv, cudaMemcpyHostToDevice);
    check_special<<<(nv * nv + 127) / 128, 128>>>(bad, dv, nv);
    total += (unsigned long long)nv * nv;
    const cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(&hbad, bad, sizeof hbad, cudaMemcpyDeviceToHost);
    printf("quotients %llu mismatches %llu (%s)\n", total, hbad, cudaGetErrorString(e));
    return (e != cudaSuccess || hbad) ? 1 : 0;
}
