// lbm_noalloc.cu -- moment reduction that performs no device allocation.
//
// Some callers cannot call cudaMalloc.  They include code running inside
// another framework's memory pool or allocation policy, hosts that forbid
// allocation after start-up (real-time or certified loops), and drivers that
// budget every byte of device memory themselves.  jlb_reduce_moments_noalloc
// serves them: it computes the same FP64 sums as jlb_reduce from arrays the
// caller owns.  Its scratch space for per-block partial sums is the static
// device array below, which each GPU that loads the library holds until the
// process exits.
#include <cuda_runtime.h>
#include <math.h>
#include <mutex>

#include "jyulb_gb300.h"
#include "lbm_common.h"

namespace {

using namespace jlb;

constexpr int NA_THREADS = 256;
constexpr int64_t NA_MAX_SITES = (int64_t)1 << 28;
constexpr int NA_MAX_PARTIALS = 4096;   // blocks of the partial-sum pass
constexpr int NA_COMPONENTS = 8;

// Partial sums of the last call: at most 4096 x 8 doubles = 256 KiB per
// device.
static __device__ __align__(256) double g_noalloc_scratch[NA_MAX_PARTIALS * NA_COMPONENTS];

template <class C, bool SHIFTED>
__global__ void __launch_bounds__(NA_THREADS) noalloc_partial_kernel(const uint32_t *nmask, const C *den,
                                                                     const C *ux, const C *uy, const C *uz,
                                                                     int64_t n_sites, double *partial) {
    double acc[NA_COMPONENTS] = {0, 0, 0, 0, 0, 0, 0, 0};
    // grid-stride: the grid is sized to the GPU, not to the input
    const int64_t stride = (int64_t)gridDim.x * NA_THREADS;
    for (int64_t n = (int64_t)blockIdx.x * NA_THREADS + threadIdx.x; n < n_sites; n += stride) {
        if (nmask[n] & MASK_SOLID) continue;
        const double d = SHIFTED ? 1.0 + (double)den[n] : (double)den[n];
        const double u0 = (double)ux[n], u1 = (double)uy[n], u2 = (double)uz[n];
        acc[0] += d;
        acc[1] += d * u0; acc[2] += d * u1; acc[3] += d * u2;
        acc[4] += u0; acc[5] += u1; acc[6] += u2;
        if (!isfinite(d) || !isfinite(u0) || !isfinite(u1) || !isfinite(u2)) acc[7] += 1.0;
    }
    __shared__ double sm[NA_COMPONENTS][NA_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NA_COMPONENTS; ++c) {
        double v = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[c][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < NA_COMPONENTS) {
        double v = 0.0;
        for (int w = 0; w < NA_THREADS / 32; ++w) v += sm[threadIdx.x][w];
        // every partial this call reads is written here first, so the
        // leftovers of earlier calls never need clearing
        partial[(int64_t)blockIdx.x * NA_COMPONENTS + threadIdx.x] = v;
    }
}

__global__ void noalloc_final_kernel(const double *partial, int nblocks, double *out) {
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (c >= NA_COMPONENTS) return;
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += partial[(int64_t)b * NA_COMPONENTS + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[c] = v;
}

// device address of the static scratch and the SM count, per device; a
// lookup is kept only once it succeeded (a failed one, e.g. under stream
// capture, is retried by the next call)
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_mu;
double *g_scratch_ptr[NA_MAX_DEVICES] = {nullptr};
int g_sms[NA_MAX_DEVICES] = {0};

bool scratch_of(int dev, double *&ptr, int &sms) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        // the host name of g_noalloc_scratch is only a stand-in for the
        // device array: resolve its device address with this device current
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError(); // leave no error of the failed lookup behind
            return false;
        }
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        g_sms[dev] = n > 0 ? n : 1;
        g_scratch_ptr[dev] = (double *)p;
    }
    ptr = g_scratch_ptr[dev];
    sms = g_sms[dev];
    return true;
}

} // namespace

extern "C" int jlb_reduce_moments_noalloc(const uint32_t *nmask, const void *den, const void *ux, const void *uy,
                                          const void *uz, int64_t n_sites, int32_t precision, double *out,
                                          void *stream) {
    if (!nmask || !den || !ux || !uy || !uz || !out) return JLB_ERR_INVALID_ARG;
    if (n_sites < 1 || n_sites > NA_MAX_SITES) return JLB_ERR_INVALID_ARG;
    if (precision != JLB_FP64 && precision != JLB_FP32 && precision != JLB_FP16) return JLB_ERR_INVALID_ARG;
    // an error left in the runtime's last-error slot by an earlier, unrelated
    // launch is not this call's failure
    cudaGetLastError();
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return JLB_ERR_CUDA; }
    if (dev < 0 || dev >= NA_MAX_DEVICES) return JLB_ERR_UNSUPPORTED;
    double *partial = nullptr;
    int sms = 1;
    if (!scratch_of(dev, partial, sms)) return JLB_ERR_CUDA;
    // four blocks per SM, fewer for inputs of fewer sites than that covers
    int64_t nb = 4 * (int64_t)sms;
    const int64_t need = (n_sites + NA_THREADS - 1) / NA_THREADS;
    if (nb > need) nb = need;
    if (nb > NA_MAX_PARTIALS) nb = NA_MAX_PARTIALS;
    const int nblocks = (int)nb;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == JLB_FP64)
        noalloc_partial_kernel<double, false><<<nblocks, NA_THREADS, 0, st>>>(
            nmask, (const double *)den, (const double *)ux, (const double *)uy, (const double *)uz, n_sites,
            partial);
    else
        noalloc_partial_kernel<float, true><<<nblocks, NA_THREADS, 0, st>>>(
            nmask, (const float *)den, (const float *)ux, (const float *)uy, (const float *)uz, n_sites,
            partial);
    if (cudaGetLastError() != cudaSuccess) return JLB_ERR_CUDA;
    noalloc_final_kernel<<<1, 256, 0, st>>>(partial, nblocks, out);
    return cudaGetLastError() == cudaSuccess ? JLB_OK : JLB_ERR_CUDA;
}
