// Integer-pipe peak of the NTT's Barrett product (bmul, common.cuh): a register-only kernel whose
// rate is the denominator of the compute-bound transforms' integer roofline. No memory traffic
// but one word per thread at the end; every chain stays within |x| <= 3n/4 (bmul's bound), so the
// work is exactly the transforms' product on in-range operands.
#include "common.cuh"

namespace {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_CHAINS = 8;  // independent products in flight per thread

__global__ void __launch_bounds__(PEAK_THREADS) barrett_peak_kernel(int64_t z, int64_t u, int64_t n, int iters,
                                                                    int64_t* out) {
    const int64_t tid = (int64_t)blockIdx.x * PEAK_THREADS + threadIdx.x;
    int64_t x[PEAK_CHAINS];
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) x[c] = (tid * 7919 + c * 104729) % n;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < PEAK_CHAINS; c++) x[c] = bmul(z, u, x[c], n);
    }
    int64_t acc = 0;
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) acc ^= x[c];
    out[tid] = acc;
}

// Int8 tensor-core rate available to this target. sm_103a has no int8 form of tcgen05.mma (ptxas:
// "Feature '.kind::i8' not supported on .target 'sm_103a'"), so the warp-level
// mma.sync.m16n8k32 s8 x s8 -> s32 instruction is the only int8 tensor path; this kernel issues
// it from registers only, MMA_CHAINS independent accumulators per warp, to measure its rate (the
// denominator of an int8 limb-split base conversion, which would need 64 int8 products per
// 57-bit x 56-bit term).
constexpr int MMA_CHAINS = 8;

__global__ void __launch_bounds__(PEAK_THREADS) int8_mma_peak_kernel(int iters, int32_t* out) {
    const uint32_t tid = blockIdx.x * PEAK_THREADS + threadIdx.x;
    uint32_t a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = (tid * 2654435761u) ^ (0x01010101u * (i + 1));
#pragma unroll
    for (int i = 0; i < 2; i++) b[i] = (tid * 40503u) ^ (0x03050709u * (i + 1));
    int32_t c[MMA_CHAINS][4];
#pragma unroll
    for (int k = 0; k < MMA_CHAINS; k++)
#pragma unroll
        for (int i = 0; i < 4; i++) c[k][i] = k + i;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < MMA_CHAINS; k++)
            asm volatile(
                "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
                "{%0, %1, %2, %3};\n"
                : "+r"(c[k][0]), "+r"(c[k][1]), "+r"(c[k][2]), "+r"(c[k][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
    }
    int32_t acc = 0;
#pragma unroll
    for (int k = 0; k < MMA_CHAINS; k++)
#pragma unroll
        for (int i = 0; i < 4; i++) acc ^= c[k][i];
    out[tid] = acc;
}

}  // namespace

extern "C" {

hc_status hc_int8_mma_peak(hc_context ctx, double* macs_per_s) {
    using namespace hc;
    if (!ctx || !macs_per_s) return fail(HC_ERR_ARG, "null argument");
    const int blocks = num_sms(ctx) * 8, iters = 4096;
    const size_t words = (size_t)blocks * PEAK_THREADS;
    cudaStream_t s = stream_of(ctx);
    int32_t* out = nullptr;
    count_alloc();
    hc_status st = cuda_check(cudaMallocAsync((void**)&out, words * 4, s), "peak buffer");
    if (st) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    st = cuda_check(cudaEventCreate(&e0), "peak event");
    if (!st) st = cuda_check(cudaEventCreate(&e1), "peak event");
    float ms = 0.f;
    if (!st) {
        int8_mma_peak_kernel<<<blocks, PEAK_THREADS, 0, s>>>(iters / 8, out);  // warm-up
        cudaEventRecord(e0, s);
        int8_mma_peak_kernel<<<blocks, PEAK_THREADS, 0, s>>>(iters, out);
        cudaEventRecord(e1, s);
        count_launch(ctx, 2);
        st = cuda_check(cudaGetLastError(), "peak kernel launch");
        if (!st) st = cuda_check(cudaEventSynchronize(e1), "peak kernel");
        if (!st) st = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "peak timing");
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    if (st) return st;
    if (ms <= 0.f) return fail(HC_ERR_CUDA, "peak kernel: no elapsed time");
    // one m16n8k32 instruction per warp and chain = 16 x 8 x 32 multiply-adds
    *macs_per_s = (double)words / 32 * MMA_CHAINS * iters * (16.0 * 8 * 32) / (ms * 1e-3);
    return HC_OK;
}

hc_status hc_barrett_peak(hc_context ctx, double* products_per_s) {
    using namespace hc;
    if (!ctx || !products_per_s) return fail(HC_ERR_ARG, "null argument");
    // a 57-bit odd modulus and one twiddle (z, u = round(-z 2^64 / n)) as the transforms use
    const int64_t n = ((int64_t)1 << 57) - 13, z = 0x123456789abcdLL % n;
    const i128 num = -((i128)z << 64);
    const int64_t u = (int64_t)((num >= 0 ? num + n / 2 : num - n / 2) / n);
    const int blocks = num_sms(ctx) * 8, iters = 4096;
    const size_t words = (size_t)blocks * PEAK_THREADS;
    cudaStream_t s = stream_of(ctx);
    int64_t* out = nullptr;
    count_alloc();
    hc_status st = cuda_check(cudaMallocAsync((void**)&out, words * 8, s), "peak buffer");
    if (st) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    st = cuda_check(cudaEventCreate(&e0), "peak event");
    if (!st) st = cuda_check(cudaEventCreate(&e1), "peak event");
    float ms = 0.f;
    if (!st) {
        barrett_peak_kernel<<<blocks, PEAK_THREADS, 0, s>>>(z, u, n, iters / 8, out);  // warm-up
        cudaEventRecord(e0, s);
        barrett_peak_kernel<<<blocks, PEAK_THREADS, 0, s>>>(z, u, n, iters, out);
        cudaEventRecord(e1, s);
        count_launch(ctx, 2);
        st = cuda_check(cudaGetLastError(), "peak kernel launch");
        if (!st) st = cuda_check(cudaEventSynchronize(e1), "peak kernel");
        if (!st) st = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "peak timing");
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    if (st) return st;
    if (ms <= 0.f) return fail(HC_ERR_CUDA, "peak kernel: no elapsed time");
    *products_per_s = (double)words * PEAK_CHAINS * iters / (ms * 1e-3);
    return HC_OK;
}

}  // extern "C"
