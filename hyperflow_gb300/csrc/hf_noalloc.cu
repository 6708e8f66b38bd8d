// hf_time_step_noalloc: the CFL time step of one block, for callers that cannot allocate.
//
// Some callers cannot call cudaMalloc: an application that hands all device memory to
// its own pool allocator up front, a solver running under a strict no-allocation rule in
// its time loop, or code driving the step from inside a region where allocation is
// forbidden.  Every other entry point of this library allocates (its context owns device
// buffers and a control block).  This one allocates nothing.  The caller passes the
// state and the output word in device memory.  The only working memory is the file-scope
// array below, fixed at load time.
//
// Limits and sharing:
//   * at most kNoAllocMaxCtas CTAs of kNoAllocCellsPerCta cells, i.e. up to
//     kNoAllocMaxCells = 16,777,216 cells (a 4096 x 4096 block with its ghosts does not
//     fit; 4094 x 4094 interior cells with 1 ghost do); larger blocks are rejected with
//     HF_ERR_TOO_LARGE before any launch;
//   * the scratch array is 64 KiB + 256 B and stays resident on every GPU that loads
//     the library until the process exits;
//   * every call uses the same array, which keeps the previous call's contents; each call
//     clears its arrival counter first (cudaMemsetAsync on the caller's stream).  Calls
//     whose kernels overlap on the GPU (different streams, or different host threads
//     without ordering) race on the array and give wrong results;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and keeps it once the lookup succeeds;
//     a lookup that fails returns HF_ERR_CUDA and is retried by the next call.  Make that
//     first call before any stream capture that includes this entry point.
#include <cstdint>
#include <mutex>

#include "../../include/hyperflow_gb300.h"
#include "hf_device.cuh"

namespace hf {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocCellsPerThread = 16;
constexpr int kNoAllocCellsPerCta = kNoAllocThreads * kNoAllocCellsPerThread;   // 4096
constexpr int kNoAllocMaxCtas = 4096;
constexpr long long kNoAllocMaxCells = (long long)kNoAllocMaxCtas * kNoAllocCellsPerCta;

// [0, 2*kNoAllocMaxCtas): per-CTA partial maxima (|u|+c, |v|+c); then the arrival counter
static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocMaxCtas + 32];

constexpr int kMaxDevices = 64;
static void* g_scratch_addr[kMaxDevices];   // set once a lookup on that device has succeeded
static std::mutex g_scratch_mutex;

// TimeStep::operator() (src/fvm_2d_cart/scheme/timestep/timestep.cpp:29-68) over every cell
// of one block, ghosts included.  Each CTA writes its two partial maxima; the last CTA to
// arrive folds them and writes the dt.
__global__ void __launch_bounds__(kNoAllocThreads)
noalloc_cfl_kernel(const double* __restrict__ U, int tx, int ty, int pitch, double dx, double dy,
                   double gamma, double final_cfl, double* __restrict__ dt_out,
                   double* __restrict__ scratch) {
    const double g1 = gamma - 1.0;
    const long long n = (long long)tx * ty;
    const size_t plane = (size_t)ty * pitch;
    double mx = 0.0, my = 0.0;
    const long long base = (long long)blockIdx.x * kNoAllocCellsPerCta;
    for (int k = 0; k < kNoAllocCellsPerThread; ++k) {
        long long c = base + (long long)k * kNoAllocThreads + threadIdx.x;
        if (c >= n) break;
        int i = (int)(c % tx), j = (int)(c / tx);
        size_t o = (size_t)j * pitch + i;
        double sx, sy;
        wave_terms(gamma, g1, U[o], U[plane + o], U[2 * plane + o], U[3 * plane + o], sx, sy);
        mx = nmax(mx, sx);
        my = nmax(my, sy);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = nmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        my = nmax(my, __shfl_xor_sync(0xffffffffu, my, o));
    }
    __shared__ double red[2][kNoAllocThreads / 32];
    __shared__ bool last;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { red[0][w] = mx; red[1][w] = my; }
    __syncthreads();
    unsigned int* arrivals = reinterpret_cast<unsigned int*>(scratch + 2 * kNoAllocMaxCtas);
    if (threadIdx.x == 0) {
        for (int k = 1; k < kNoAllocThreads / 32; ++k) {
            mx = nmax(mx, red[0][k]);
            my = nmax(my, red[1][k]);
        }
        scratch[2 * blockIdx.x] = mx;
        scratch[2 * blockIdx.x + 1] = my;
        __threadfence();
        last = (atomicAdd(arrivals, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    volatile double* vs = scratch;
    double ax = 0.0, ay = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) {
        ax = nmax(ax, vs[2 * b]);
        ay = nmax(ay, vs[2 * b + 1]);
    }
    // fl(dx / s) is non-increasing in s, so min over cells of dx / s = dx / max s
    double dtx = smin(1e16, dx / ax);
    double dty = smin(1e16, dy / ay);
    *dt_out = final_cfl * smin(dtx, dty);
    *arrivals = 0u;
}

}  // namespace hf

extern "C" int hf_time_step_noalloc(const double* d_cons, int total_x, int total_y, int pitch,
                                    double dx, double dy, double gamma, double cfl,
                                    int64_t call_index, double* d_dt, void* stream) {
    using namespace hf;
    if (!d_cons || !d_dt || total_x <= 0 || total_y <= 0 || pitch < total_x || call_index < 0)
        return HF_ERR_ARG;
    const long long n = (long long)total_x * total_y;
    if (n > kNoAllocMaxCells) return HF_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HF_ERR_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return HF_ERR_ARG;
    // the array's device address, looked up with this device current and kept once the lookup
    // has succeeded; a failed lookup (say, made inside a stream capture) is not kept, so a
    // later call retries it
    double* scratch;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void* addr = nullptr;
            if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) {
                (void)cudaGetLastError();   // clear the failed call's error state
                return HF_ERR_CUDA;
            }
            g_scratch_addr[dev] = addr;
        }
        scratch = static_cast<double*>(g_scratch_addr[dev]);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(scratch + 2 * kNoAllocMaxCtas, 0, sizeof(unsigned int), s) != cudaSuccess)
        return HF_ERR_CUDA;
    const int grid = (int)((n + kNoAllocCellsPerCta - 1) / kNoAllocCellsPerCta);
    // TimeStep's start-up multiplier (timestep.cpp:60-66): 0.2 for the first 10 calls
    const double final_cfl = (call_index + 1 <= 10) ? 0.2 * cfl : cfl;
    noalloc_cfl_kernel<<<grid, kNoAllocThreads, 0, s>>>(d_cons, total_x, total_y, pitch, dx, dy,
                                                         gamma, final_cfl, d_dt, scratch);
    return cudaGetLastError() == cudaSuccess ? HF_OK : HF_ERR_CUDA;
}
