// Issue-rate microbenchmarks used as roofline denominators that the driver's
// MEASURED_PEAKS.json does not hold: FP64 FFMA, FP32 FFMA, FP64 mma.sync
// (m8n8k4), and mma.sync TF32 m16n8k8 / BF16 m16n8k16. Register-only loops;
// each thread writes one value (buffer sized to the grid).
#include "engine.h"

namespace itg {

template <typename T>
__global__ void peak_ffma_kernel(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
            x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void peak_dmma_kernel(double* out, int iters) {
    double a = threadIdx.x * 1e-3, b = 1.0 + threadIdx.x * 1e-4;
    double c[4][2] = {};
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 4; j++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};"
                         : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = c[0][0] + c[1][0] + c[2][0] + c[3][0] + c[0][1] + c[1][1] + c[2][1] + c[3][1];
}

__global__ void peak_tf32_kernel(float* out, int iters) {
    unsigned a0 = __float_as_uint(1.0f + threadIdx.x), b0 = __float_as_uint(0.5f);
    float c[4][4] = {};
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 4; j++)
            asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                         : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                         : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
    }
    float s = 0;
    for (int j = 0; j < 4; j++) for (int k = 0; k < 4; k++) s += c[j][k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void peak_bf16_kernel(float* out, int iters) {
    unsigned a0 = 0x3f803f80u + threadIdx.x, b0 = 0x3f003f00u;
    float c[4][4] = {};
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 4; j++)
            asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                         : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                         : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
    }
    float s = 0;
    for (int j = 0; j < 4; j++) for (int k = 0; k < 4; k++) s += c[j][k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// TFLOP/s of [fp64 ffma, fp32 ffma, fp64 mma.sync, tf32 mma.sync, bf16 mma.sync]
void measure_peaks(Ctx& ctx, double* tflops) {
    const int threads = 256, blocks = ctx.sm_count * 8;
    const size_t n = (size_t)threads * blocks;
    DevBuf buf(n * sizeof(double), ctx.stream);
    cudaEvent_t e0, e1;
    ITG_CHECK_CUDA(cudaEventCreate(&e0));
    ITG_CHECK_CUDA(cudaEventCreate(&e1));
    auto time = [&](auto launch, double flops) {
        launch(4);  // warm
        ITG_CHECK_CUDA(cudaEventRecord(e0, ctx.stream));
        launch(0);
        ITG_CHECK_CUDA(cudaEventRecord(e1, ctx.stream));
        ITG_CHECK_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        ITG_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return flops / (ms * 1e-3) / 1e12;
    };
    const int it64 = 1000, it32 = 20000, itm = 1000, itt = 10000;
    tflops[0] = time([&](int w) { peak_ffma_kernel<double><<<blocks, threads, 0, ctx.stream>>>(buf.as<double>(), w ? w : it64, 1.0000001, 1e-9); },
                     2.0 * 64 * it64 * (double)n);
    tflops[1] = time([&](int w) { peak_ffma_kernel<float><<<blocks, threads, 0, ctx.stream>>>(buf.as<float>(), w ? w : it32, 1.0000001f, 1e-9f); },
                     2.0 * 64 * it32 * (double)n);
    tflops[2] = time([&](int w) { peak_dmma_kernel<<<blocks, threads, 0, ctx.stream>>>(buf.as<double>(), w ? w : itm); },
                     2.0 * 8 * 8 * 4 * 4.0 * itm * (n / 32));
    tflops[3] = time([&](int w) { peak_tf32_kernel<<<blocks, threads, 0, ctx.stream>>>(buf.as<float>(), w ? w : itt); },
                     2.0 * 16 * 8 * 8 * 4.0 * itt * (n / 32));
    tflops[4] = time([&](int w) { peak_bf16_kernel<<<blocks, threads, 0, ctx.stream>>>(buf.as<float>(), w ? w : itt); },
                     2.0 * 16 * 8 * 16 * 4.0 * itt * (n / 32));
    ITG_CHECK_CUDA(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

}  // namespace itg
