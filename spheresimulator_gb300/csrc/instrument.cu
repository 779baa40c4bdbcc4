// instrument.cu — measurement helpers exported for benchmarks: the FP32 and FP64 FMA issue rates
// of the device (independent FMA chains, no memory traffic). These are the SIMT roofline
// denominators of the all-pairs far field, measured on the same GPU in the same run.
#include <cuda_runtime.h>

#include "../../include/smob.h"

namespace {

template <typename T>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
    T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i) {
        x0 = x0 * a + b;
        x1 = x1 * a + b;
        x2 = x2 * a + b;
        x3 = x3 * a + b;
        x4 = x4 * a + b;
        x5 = x5 * a + b;
        x6 = x6 * a + b;
        x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double measure(int sms, int iters) {
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double best = 0;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(a);
        k_fma_chain<T><<<blocks, threads>>>(out, iters, T(0.999), T(1e-3));
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        const double tf = 2.0 * 8 * double(iters) * blocks * threads / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    return best;
}

}  // namespace

extern "C" smob_status smob_measure_fma_peaks(int device, double* fp32_tflops, double* fp64_tflops) {
    if (cudaSetDevice(device) != cudaSuccess) return SMOB_ERR_NO_DEVICE;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (fp32_tflops) *fp32_tflops = measure<float>(sms, 1 << 16);
    if (fp64_tflops) *fp64_tflops = measure<double>(sms, 1 << 12);
    return cudaGetLastError() == cudaSuccess ? SMOB_OK : SMOB_ERR_CUDA;
}
