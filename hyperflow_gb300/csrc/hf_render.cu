// Frame images: the "schlieren-like" normalised exponentiated gradient of the reference's
// plotting script (src/visualisation/euler/euler_2d.py:214-295) and a linear grey map, on the
// GPU.  C ABI in include/hyperflow_gb300_render.h.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/hyperflow_gb300_render.h"
#include "hf_device.cuh"

namespace hf {

constexpr int kRenderNT = 256;

// [0] max |grad| (bit pattern of a non-negative double), [1] min / [2] max of the imaged field
// as order-preserving keys, [3] nonzero once an interior gradient that is a number was seen
__device__ unsigned long long g_render_red[4];

// a double's bits mapped so that unsigned order is numeric order (NaN excluded by the callers)
__device__ __forceinline__ unsigned long long range_key(double x) {
    const unsigned long long b = dbits(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_range_key(unsigned long long k) {
    return bitsd((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k);
}

__global__ void render_reset_kernel() {
    g_render_red[0] = 0ull;
    g_render_red[1] = ~0ull;
    g_render_red[2] = 0ull;
    g_render_red[3] = 0ull;
}

// |grad f| by central differences over the interior cells (euler_2d.py:252-284; the one-sided
// branches there are never taken, the loops skipping the boundary cells, whose value stays 0),
// and its maximum (NaN cells excluded, as the reference's comparisons exclude them)
__global__ void __launch_bounds__(kRenderNT) render_grad_kernel(const double* __restrict__ f, int nx, int ny,
                                                               double dx, double dy, double* __restrict__ g) {
    double mx = 0.0;
    int seen = 0;
    const long long n = (long long)nx * ny;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % nx), j = (int)(k / nx);
        double v = 0.0;
        if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1) {
            const double divx = (f[k + 1] - f[k - 1]) / (2.0 * dx);
            const double divy = (f[k + nx] - f[k - nx]) / (2.0 * dy);
            v = sqrt(divx * divx + divy * divy);
            mx = nmax(mx, v);
            seen |= v == v;
        }
        g[k] = v;
    }
    if (__any_sync(0xffffffffu, seen) && (threadIdx.x & 31) == 0) atomicOr(&g_render_red[3], 1ull);
    block_max2_atomic<kRenderNT>(mx, 0.0, &g_render_red[0], &g_render_red[0]);
}

// s = beta * exp(-lambda * |grad| / max |grad|) (euler_2d.py:288-293); the maximum starts at
// -1e6 there, which is what remains when no interior gradient is a number
__global__ void __launch_bounds__(kRenderNT) render_exp_kernel(double* __restrict__ g, long long n, double beta,
                                                              double lambda) {
    const double gmax = g_render_red[3] ? bitsd(g_render_red[0]) : -1e6;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        g[k] = beta * exp(-lambda * g[k] / gmax);
}

__global__ void __launch_bounds__(kRenderNT) render_range_kernel(const double* __restrict__ v, long long n) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const double x = v[k];
        if (x == x && fabs(x) <= 1.7976931348623157e308) {   // finite
            const unsigned long long key = range_key(x);
            lo = key < lo ? key : lo;
            hi = key > hi ? key : hi;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        if (lo != ~0ull) atomicMin(&g_render_red[1], lo);
        if (hi != 0ull) atomicMax(&g_render_red[2], hi);
    }
}

__global__ void __launch_bounds__(kRenderNT) render_image_kernel(const double* __restrict__ v, long long n, int fixed,
                                                                double lo_in, double hi_in,
                                                                unsigned char* __restrict__ img) {
    double lo = lo_in, hi = hi_in;
    if (!fixed) {
        lo = g_render_red[1] == ~0ull ? 0.0 : from_range_key(g_render_red[1]);
        hi = g_render_red[2] == 0ull ? 1.0 : from_range_key(g_render_red[2]);
    }
    const double span = hi > lo ? hi - lo : 1.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const double x = v[k];
        unsigned char c = 0;
        if (x == x) {
            double t = (x - lo) / span;
            t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
            c = (unsigned char)floor(255.0 * t + 0.5);
        }
        img[k] = c;
    }
}

}  // namespace hf

extern "C" int hf_render_gray(const double* d_field, int nx, int ny, double dx, double dy, int schlieren,
                              double beta, double lambda, const double* limits, double* d_out,
                              unsigned char* d_image, void* stream) {
    if (!d_field || !d_image || nx < 1 || ny < 1 || (schlieren && !d_out)) return HF_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long n = (long long)nx * ny;
    long long want = (n + hf::kRenderNT - 1) / hf::kRenderNT;
    const int grid = (int)(want > 8 * 152 ? 8 * 152 : want);
    hf::render_reset_kernel<<<1, 1, 0, s>>>();
    const double* v = d_field;
    if (schlieren) {
        hf::render_grad_kernel<<<grid, hf::kRenderNT, 0, s>>>(d_field, nx, ny, dx, dy, d_out);
        hf::render_exp_kernel<<<grid, hf::kRenderNT, 0, s>>>(d_out, n, beta, lambda);
        v = d_out;
    } else if (d_out) {
        if (cudaMemcpyAsync(d_out, d_field, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return HF_ERR_CUDA;
        v = d_out;
    }
    if (!limits) hf::render_range_kernel<<<grid, hf::kRenderNT, 0, s>>>(v, n);
    hf::render_image_kernel<<<grid, hf::kRenderNT, 0, s>>>(v, n, limits ? 1 : 0, limits ? limits[0] : 0.0,
                                                           limits ? limits[1] : 1.0, d_image);
    return cudaGetLastError() == cudaSuccess ? HF_OK : HF_ERR_CUDA;
}
