// k_probe.cu -- FP64/FP32 FMA throughput of this GPU (the ALU denominators
// of the FP64 stencil and wavelet rooflines). A measurement helper, built as
// its own library (libwg_probe.so) beside the product library and loaded only
// by the benchmark.
#include <cuda_runtime.h>

namespace wg {

template <class T>
__global__ void __launch_bounds__(256) fma_chain(T *out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
static cudaError_t probe_one(int iters, double *tflops) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int blocks = sms * 16, threads = 256;
    T *out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(T) * blocks * threads);
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0);
        fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    e = cudaGetLastError();
    *tflops = 2.0 * 8 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return e;
}

}  // namespace wg

// FP64 and FP32 FMA throughput of the current device in TFLOP/s (FMA = 2);
// 0 on success, else the CUDA error code.
extern "C" int wg_probe_alu(double *fp64_tflops, double *fp32_tflops) {
    if (!fp64_tflops || !fp32_tflops) return (int)cudaErrorInvalidValue;
    cudaError_t e = wg::probe_one<double>(2048, fp64_tflops);
    if (e == cudaSuccess) e = wg::probe_one<float>(16384, fp32_tflops);
    return (int)e;
}
