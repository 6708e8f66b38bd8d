// Self-tests of device arithmetic against the hardware (declared in
// include/hyperflow_gb300_diag.h): the integer-pipe division must reproduce the IEEE
// division bit for bit on every input.
#include <cstdint>

#include "../../include/hyperflow_gb300_diag.h"
#include "hf_intdiv.cuh"

namespace hf {

__device__ __forceinline__ uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double mk(uint64_t sign, uint64_t exp, uint64_t mant) {
    return __longlong_as_double((long long)((sign << 63) | ((exp & 0x7FF) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// division -- mode 0: raw random bit patterns; 1: normal operands, exponent difference within
// +-80; 2: near-halfway quotients (a = q*b rounded, mantissas perturbed by a few units);
// 3: short mantissas (exact and near-exact quotients); 4: operands near the range limits.
// square root -- mode 5: raw bit patterns; 6: every normal exponent; 7: near-squares.
__global__ void div_check_kernel(uint64_t seed, long long n, int mode, unsigned long long* bad,
                                 double* first) {
    uint64_t s = seed ^ (0x1234567ull * (blockIdx.x * blockDim.x + threadIdx.x + 1));
    const bool sq = mode >= 5;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        uint64_t r1 = splitmix(s), r2 = splitmix(s), r3 = splitmix(s);
        double a, b;
        if (mode == 0 || mode == 5) {
            a = __longlong_as_double((long long)r1);
            b = __longlong_as_double((long long)r2);
        } else if (mode == 1) {
            uint64_t eb = 1023 - 200 + (r3 % 400), ea = eb + (int64_t)((r3 >> 20) % 161) - 80;
            a = mk(r1 >> 63, ea, r1);
            b = mk(r2 >> 63, eb, r2);
        } else if (mode == 2) {
            b = mk(0, 1023 + (r3 % 64) - 32, r2);
            double q = mk(r3 >> 63, 1023 + ((r3 >> 8) % 16) - 8, r1);
            a = __dmul_rn(q, b);
            long long ab = __double_as_longlong(a) + (long long)((r3 >> 20) % 7) - 3;
            a = __longlong_as_double(ab);
        } else if (mode == 3) {
            a = mk(0, 1023 + (r3 % 30), (r1 >> 40) << 40);
            b = mk(r2 >> 63, 1023 + ((r3 >> 8) % 30), (r2 >> 44) << 44);
        } else if (mode == 4) {
            uint64_t e1 = (r3 & 1) ? 1 + (r3 >> 1) % 60 : 2046 - (r3 >> 1) % 60;
            uint64_t e2 = (r3 & 2) ? 1 + (r3 >> 8) % 60 : 2046 - (r3 >> 8) % 60;
            a = mk(r1 >> 63, e1, r1);
            b = mk(r2 >> 63, e2, r2);
        } else {     // 6, 7: sqrt arguments built below
            a = mk(0, 1023 + (r3 % 40) - 20, r1);
            b = 1.0;
        }
        double got, want;
        if (sq) {
            a = mode == 5 ? a : (mode == 6 ? mk(0, 1 + r3 % 2046, r1) : a * a);
            if (mode == 7) a = __longlong_as_double(__double_as_longlong(a) + (long long)((r3 >> 40) % 5) - 2);
            got = sqrt_rn(a);
            want = __dsqrt_rn(a);
            b = 0.0;
        } else {
            got = div_rn(a, b);
            want = __ddiv_rn(a, b);
        }
        const bool same = (__double_as_longlong(got) == __double_as_longlong(want)) || (got != got && want != want);
        if (!same) {
            unsigned long long i = atomicAdd(bad, 1ull);
            if (i == 0) { first[0] = a; first[1] = b; first[2] = got; first[3] = want; }
        }
    }
}

}  // namespace hf

extern "C" int hf_diag_div_check(uint64_t seed, int64_t n, int mode, int64_t* mismatches, double* first4) {
    if (!mismatches || n < 0 || mode < 0 || mode > 7) return HF_ERR_ARG;
    unsigned long long* dbad = nullptr;
    double* dfirst = nullptr;
    if (cudaMalloc(&dbad, sizeof(unsigned long long)) != cudaSuccess) return HF_ERR_CUDA;
    if (cudaMalloc(&dfirst, 4 * sizeof(double)) != cudaSuccess) { cudaFree(dbad); return HF_ERR_CUDA; }
    cudaMemset(dbad, 0, sizeof(unsigned long long));
    cudaMemset(dfirst, 0, 4 * sizeof(double));
    hf::div_check_kernel<<<152 * 8, 256>>>(seed, n, mode, dbad, dfirst);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h = 0;
    double f[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) {
        cudaMemcpy(&h, dbad, sizeof h, cudaMemcpyDeviceToHost);
        cudaMemcpy(f, dfirst, sizeof f, cudaMemcpyDeviceToHost);
    }
    cudaFree(dbad);
    cudaFree(dfirst);
    if (e != cudaSuccess) return HF_ERR_CUDA;
    *mismatches = (int64_t)h;
    if (first4)
        for (int k = 0; k < 4; ++k) first4[k] = f[k];
    return HF_OK;
}
