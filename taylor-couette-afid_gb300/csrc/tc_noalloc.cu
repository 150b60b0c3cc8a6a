// tc_noalloc.cu -- tc_check_divergence_noalloc: CheckDivergence.F90:28-43 on
// velocity arrays the caller keeps on the device, in the reference layout,
// without allocating anything.
//
// The kernels are the two-pass maximum of tc_check_divergence (per-block
// maxima, then one finishing block); the difference is where the scratch
// lives.  Here it is one file-scope __device__ array:
//   [0, kNaMaxR)             udx2m(1:nrm), copied from the caller's host array
//   [kNaMaxR, 2 kNaMaxR)     usrm(1:nrm)
//   [2 kNaMaxR, +kNaBlocks)  per-block maxima
//   [2 kNaMaxR + kNaBlocks]  the result
// 16,689 doubles (130 KB) per device.  Nothing in it has to start at zero:
// every call writes the coefficients and every per-block slot before it
// reads them.  Its address is looked up once per device with
// cudaGetSymbolAddress, by the first call made with that device current.
// All calls on one device share the array, so calls must not overlap.
// A NaN anywhere in the fields makes the result NaN and the status 169.

#include <cmath>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/tc_capi.h"

namespace tcgb {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kNaMaxR = 8192;      // radial cells the scratch holds
constexpr int kNaBlocks = 304;     // 2 x 152 SMs
constexpr int kNaThreads = 256;
constexpr int kNaMaxDevices = 64;
constexpr int kNaWords = 2 * kNaMaxR + kNaBlocks + 1;

static __device__ __align__(256) double g_noalloc_scratch[kNaWords];

std::mutex g_na_mutex;
double* g_na_addr[kNaMaxDevices] = {nullptr};

// A maximum that keeps a NaN (fmax would drop it), so that a field that has
// blown up reports NaN instead of the largest finite divergence.
__device__ __forceinline__ double na_max(double a, double b) { return (b != b || b > a) ? b : a; }

__device__ __forceinline__ double na_warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = na_max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ double na_block_max(double v) {
    __shared__ double sh[32];
    v = na_warp_max(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        v = na_warp_max(v);
    }
    return v;
}

// |div| of every cell (k, j, i), k = 1..nrm, j = 1..nzm, i = 1..nthm, read
// from q(1:nr, 0:nzm+1, 0:nthm+1) with r fastest; the theta and z neighbours
// at i = nthm and j = nzm come from the halo, as in the reference.
__global__ void __launch_bounds__(kNaThreads) na_divmax_kernel(const double* __restrict__ qt,
                                                                const double* __restrict__ qr,
                                                                const double* __restrict__ qz, int nthm, int nzm,
                                                                int nrm, double dxt, double dxz,
                                                                double* __restrict__ scratch) {
    const int nr = nrm + 1;
    const size_t sj = (size_t)nr, si = (size_t)nr * (nzm + 2);
    const double* udx2m = scratch;
    const double* usrm = scratch + kNaMaxR;
    const long long n = (long long)nrm * nzm * nthm;
    double best = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % nrm);
        const long long rest = t / nrm;
        const int j = (int)(rest % nzm) + 1, i = (int)(rest / nzm) + 1;
        const size_t o = (size_t)k + (size_t)j * sj + (size_t)i * si;
        const double t0 = __ldg(qt + o), t1 = __ldg(qt + o + si);
        const double r0 = __ldg(qr + o), r1 = __ldg(qr + o + 1);
        const double z0 = __ldg(qz + o), z1 = __ldg(qz + o + sj);
        const double v = fabs(((t1 - t0) * dxt + (r1 - r0) * udx2m[k]) * usrm[k] + (z1 - z0) * dxz);
        best = na_max(best, v);
    }
    best = na_block_max(best);
    if (threadIdx.x == 0) scratch[2 * kNaMaxR + blockIdx.x] = best;
}

__global__ void __launch_bounds__(kNaThreads) na_finish_kernel(double* scratch) {
    double best = 0.0;
    for (int t = threadIdx.x; t < kNaBlocks; t += blockDim.x) best = na_max(best, scratch[2 * kNaMaxR + t]);
    best = na_block_max(best);
    if (threadIdx.x == 0) scratch[2 * kNaMaxR + kNaBlocks] = best;
}

int na_fail(int code, const std::string& msg) {
    tcgb::set_last_error(msg);
    return code;
}

int na_cuda(cudaError_t c, const char* what) {
    return na_fail(1000 + (int)c, std::string("tc_check_divergence_noalloc: ") + what + ": " + cudaGetErrorString(c));
}

}  // namespace

// Declared extern "C" in tc_capi.h.
int tc_check_divergence_noalloc(const double* qt, const double* qr, const double* qz, int nthm, int nzm, int nrm,
                                const double* udx2m, const double* usrm, double dxt, double dxz, void* stream,
                                double* qmax) {
    if (!qt || !qr || !qz || !udx2m || !usrm || !qmax)
        return na_fail(2000, "tc_check_divergence_noalloc: null argument");
    if (nthm < 1 || nzm < 1 || nrm < 1) return na_fail(2016, "tc_check_divergence_noalloc: nthm, nzm and nrm must be >= 1");
    if (nrm > kNaMaxR)
        return na_fail(2016, "tc_check_divergence_noalloc: nrm = " + std::to_string(nrm) + " exceeds the " +
                                 std::to_string(kNaMaxR) + " radial cells its static scratch holds");
    int dev = 0;
    cudaError_t c = cudaGetDevice(&dev);
    if (c != cudaSuccess) return na_cuda(c, "cudaGetDevice");
    if (dev < 0 || dev >= kNaMaxDevices)
        return na_fail(2016, "tc_check_divergence_noalloc: device index above " + std::to_string(kNaMaxDevices - 1));
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_addr[dev]) {
            void* p = nullptr;
            c = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (c != cudaSuccess) return na_cuda(c, "cudaGetSymbolAddress");
            g_na_addr[dev] = static_cast<double*>(p);
        }
        scratch = g_na_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The call copies from pageable host memory and synchronises the stream,
    // neither of which a stream capture allows: refuse before enqueueing.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    c = cudaStreamIsCapturing(s, &cap);
    if (c != cudaSuccess) return na_cuda(c, "cudaStreamIsCapturing");
    if (cap != cudaStreamCaptureStatusNone)
        return na_fail(2018, "tc_check_divergence_noalloc: the stream is being captured; call it outside capture");
    const size_t cb = sizeof(double) * (size_t)nrm;
    c = cudaMemcpyAsync(scratch, udx2m, cb, cudaMemcpyHostToDevice, s);
    if (c == cudaSuccess) c = cudaMemcpyAsync(scratch + kNaMaxR, usrm, cb, cudaMemcpyHostToDevice, s);
    if (c != cudaSuccess) return na_cuda(c, "coefficient copy");
    na_divmax_kernel<<<kNaBlocks, kNaThreads, 0, s>>>(qt, qr, qz, nthm, nzm, nrm, dxt, dxz, scratch);
    na_finish_kernel<<<1, kNaThreads, 0, s>>>(scratch);
    c = cudaGetLastError();
    if (c != cudaSuccess) return na_cuda(c, "launch");
    double v = 0.0;
    c = cudaMemcpyAsync(&v, scratch + 2 * kNaMaxR + kNaBlocks, sizeof v, cudaMemcpyDeviceToHost, s);
    if (c == cudaSuccess) c = cudaStreamSynchronize(s);
    if (c != cudaSuccess) return na_cuda(c, "result read");
    *qmax = v;
    if (v != v) return na_fail(169, "tc_check_divergence_noalloc: the velocity field holds a NaN");
    return 0;
}
