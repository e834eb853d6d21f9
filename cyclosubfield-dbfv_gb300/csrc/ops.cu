// Pointwise, contraction, correction and permutation kernels of the Backend trait
// (cyclosubfield-dbfv/src/hal/cpu.rs:591-1122). Every kernel walks the destination as
// (line, l) with l the contiguous dimension 3; sources are broadcast through zero strides.
#include "common.cuh"

namespace {

enum PwOp {
    OP_ASSIGN,
    OP_ASSIGN_NARROW,
    OP_ASSIGN_I128,
    OP_ADD_I64,
    OP_SUB_I64,
    OP_ADD_I128,
    OP_FMA_I64,
    OP_MUL_I64,
    OP_MUL_MONT,
    OP_ADD_RED_DOUBLE,
    OP_RED_DOUBLE,
    OP_ADD_RED,
    OP_RED,
    OP_I128_TO_MONT,
    OP_I64_TO_MONT,
};

template <int OP>
__device__ __forceinline__ void pw_apply(const KView& d, const KView& a, const KView& b, const KMods& m, int64_t i,
                                         int64_t j, int64_t k, int64_t l) {
    if (OP == OP_ASSIGN) {
        *kat<int64_t>(d, i, j, k, l) = *kat<int64_t>(a, i, j, k, l);
    } else if (OP == OP_ASSIGN_NARROW) {
        *kat<int64_t>(d, i, j, k, l) = kat<longlong2>(a, i, j, k, l)->x;  // low word of the i128
    } else if (OP == OP_ASSIGN_I128) {
        *kat<longlong2>(d, i, j, k, l) = *kat<longlong2>(a, i, j, k, l);
    } else if (OP == OP_ADD_I64) {
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        *p = wadd(*p, *kat<int64_t>(a, i, j, k, l));
    } else if (OP == OP_SUB_I64) {
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        *p = wsub(*p, *kat<int64_t>(a, i, j, k, l));
    } else if (OP == OP_ADD_I128) {
        longlong2* p = kat<longlong2>(d, i, j, k, l);
        st128(p, (i128)((u128)ld128(p) + (u128)ld128(kat<longlong2>(a, i, j, k, l))));
    } else if (OP == OP_FMA_I64 || OP == OP_MUL_I64) {
        longlong2* p = kat<longlong2>(d, i, j, k, l);
        i128 prod = (i128)*kat<int64_t>(a, i, j, k, l) * (i128)*kat<int64_t>(b, i, j, k, l);
        st128(p, OP == OP_FMA_I64 ? (i128)((u128)ld128(p) + (u128)prod) : prod);
    } else if (OP == OP_MUL_MONT) {
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        *p = mul_mont(*p, *kat<int64_t>(a, i, j, k, l), m.n[j], m.ninv[j]);
    } else if (OP == OP_ADD_RED_DOUBLE || OP == OP_RED_DOUBLE) {
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        int64_t r = double_red128(ld128(kat<longlong2>(a, i, j, k, l)), m.n[j], m.ninv[j]);
        *p = OP == OP_RED_DOUBLE ? r : wadd(*p, r);
    } else if (OP == OP_ADD_RED || OP == OP_RED) {
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        int64_t r = red128(ld128(kat<longlong2>(a, i, j, k, l)), m.n[j], m.ninv[j]);
        *p = OP == OP_RED ? r : wadd(*p, r);
    } else if (OP == OP_I128_TO_MONT) {
        *kat<int64_t>(d, i, j, k, l) = to_mont128(ld128(kat<longlong2>(a, i, j, k, l)), m.n[j], m.ninv[j], m.r3[j]);
    } else if (OP == OP_I64_TO_MONT) {
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        *p = to_mont64(*p, m.n[j], m.ninv[j], m.r2[j]);
    }
}

template <int OP>
__global__ void __launch_bounds__(256) pw_kernel(KView d, KView a, KView b, KMods m, int64_t lines, int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, r = line / d.n2;
        int64_t j = r % d.n1, i = r / d.n1;
        pw_apply<OP>(d, a, b, m, i, j, k, l);
    }
}

/// pw_kernel over a 2-D grid: blockIdx.y is the destination line (i, j, k), decomposed once per
/// thread with 32-bit arithmetic, and each thread walks LINE_SPAN / 256 positions of it, so that
/// the per-element work is the operation itself (the tile form pays several 64-bit divisions per
/// element). Used while the line count fits the grid's y dimension.
constexpr int LINE_SPAN = 1024;

template <int OP>
__global__ void __launch_bounds__(256) pw_line_kernel(KView d, KView a, KView b, KMods m) {
    const int line = (int)blockIdx.y;
    const int k = line % (int)d.n2, r = line / (int)d.n2;
    const int j = r % (int)d.n1, i = r / (int)d.n1;
    const int64_t l0 = (int64_t)blockIdx.x * LINE_SPAN;
    const int64_t l1 = l0 + LINE_SPAN < d.n3 ? l0 + LINE_SPAN : d.n3;
    for (int64_t l = l0 + threadIdx.x; l < l1; l += 256) pw_apply<OP>(d, a, b, m, i, j, k, l);
}

/// dst[i,j,k,l] = sum_u lhs[li,j,u,0] * rhs[ri,u,k,l] (src/hal/cpu.rs:791-818), i128 wrapping.
/// Four output rows j per pass share each rhs load (the matrix entries are warp-uniform loads),
/// and columns whose four entries are zero are skipped (a gadget conversion matrix is zero outside
/// each digit's columns); the sums are the same wrapping sums.
__global__ void __launch_bounds__(256) matmul_kernel(KView d, KView lhs, KView rhs, int64_t U, int64_t lines,
                                                     int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;  // (i, k)
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, i = line / d.n2;
        int64_t j = 0;
        for (; j + 4 <= d.n1; j += 4) {
            i128 acc[4] = {0, 0, 0, 0};
            for (int64_t u = 0; u < U; u++) {
                int64_t c[4];
#pragma unroll
                for (int q = 0; q < 4; q++) c[q] = *kat<int64_t>(lhs, i, j + q, u, 0);
                if ((c[0] | c[1] | c[2] | c[3]) == 0) continue;  // zero columns (a gadget matrix's) add nothing
                const int64_t x = *kat<int64_t>(rhs, i, u, k, l);
#pragma unroll
                for (int q = 0; q < 4; q++) acc[q] = (i128)((u128)acc[q] + (u128)((i128)c[q] * (i128)x));
            }
#pragma unroll
            for (int q = 0; q < 4; q++) st128(kat<longlong2>(d, i, j + q, k, l), acc[q]);
        }
        for (; j < d.n1; j++) {
            i128 acc = 0;
            for (int64_t u = 0; u < U; u++) {
                int64_t c = *kat<int64_t>(lhs, i, j, u, 0);
                int64_t x = *kat<int64_t>(rhs, i, u, k, l);
                acc = (i128)((u128)acc + (u128)((i128)c * (i128)x));
            }
            st128(kat<longlong2>(d, i, j, k, l), acc);
        }
    }
}

struct Terms {
    KView l[HC_MAX_TERMS];
    KView r[HC_MAX_TERMS];
    int n;
};

/// dst = sum_t lhs[t] * rhs[t], overwriting (src/hal/cpu.rs:707-788).
__global__ void __launch_bounds__(256) inner_product_kernel(KView d, Terms terms, int64_t lines, int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, r = line / d.n2;
        int64_t j = r % d.n1, i = r / d.n1;
        i128 acc = 0;
        for (int t = 0; t < terms.n; t++) {
            i128 prod = (i128)*kat<int64_t>(terms.l[t], i, j, k, l) * (i128)*kat<int64_t>(terms.r[t], i, j, k, l);
            acc = (i128)((u128)acc + (u128)prod);
        }
        st128(kat<longlong2>(d, i, j, k, l), acc);
    }
}

/// inner_product_kernel over the line grid of pw_line_kernel.
__global__ void __launch_bounds__(256) inner_product_line_kernel(KView d, Terms terms) {
    const int line = (int)blockIdx.y;
    const int k = line % (int)d.n2, r = line / (int)d.n2;
    const int j = r % (int)d.n1, i = r / (int)d.n1;
    const int64_t l0 = (int64_t)blockIdx.x * LINE_SPAN;
    const int64_t l1 = l0 + LINE_SPAN < d.n3 ? l0 + LINE_SPAN : d.n3;
    for (int64_t l = l0 + threadIdx.x; l < l1; l += 256) {
        i128 acc = 0;
        for (int t = 0; t < terms.n; t++) {
            i128 prod = (i128)*kat<int64_t>(terms.l[t], i, j, k, l) * (i128)*kat<int64_t>(terms.r[t], i, j, k, l);
            acc = (i128)((u128)acc + (u128)prod);
        }
        st128(kat<longlong2>(d, i, j, k, l), acc);
    }
}

/// dst[i,j,k,l] += red(((lhs[i,0,k,l] + 2^(shift-1)) >> shift) * rhs[ri,j,0,0])
/// (src/hal/cpu.rs:950-980)
__global__ void __launch_bounds__(256) bconv_correct_kernel(KView d, KView lhs, KView rhs, KMods m, int shift,
                                                            int64_t lines, int chunks) {
    const i128 half = (i128)1 << (shift - 1);
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, r = line / d.n2;
        int64_t j = r % d.n1, i = r / d.n1;
        i128 x = ld128(kat<longlong2>(lhs, i, 0, k, l));
        int64_t q = (int64_t)((i128)((u128)x + (u128)half) >> shift);
        int64_t c = *kat<int64_t>(rhs, i, j, 0, 0);
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        *p = wadd(*p, mul_mont(q, c, m.n[j], m.ninv[j]));
    }
}

/// bconv_correct_kernel over the line grid of pw_line_kernel.
__global__ void __launch_bounds__(256) bconv_correct_line_kernel(KView d, KView lhs, KView rhs, KMods m, int shift) {
    const i128 half = (i128)1 << (shift - 1);
    const int line = (int)blockIdx.y;
    const int k = line % (int)d.n2, r = line / (int)d.n2;
    const int j = r % (int)d.n1, i = r / (int)d.n1;
    const int64_t c = *kat<int64_t>(rhs, i, j, 0, 0);
    const int64_t n = m.n[j], ninv = m.ninv[j];
    const int64_t l0 = (int64_t)blockIdx.x * LINE_SPAN;
    const int64_t l1 = l0 + LINE_SPAN < d.n3 ? l0 + LINE_SPAN : d.n3;
    for (int64_t l = l0 + threadIdx.x; l < l1; l += 256) {
        i128 x = ld128(kat<longlong2>(lhs, i, 0, k, l));
        int64_t q = (int64_t)((i128)((u128)x + (u128)half) >> shift);
        int64_t* p = kat<int64_t>(d, i, j, k, l);
        *p = wadd(*p, mul_mont(q, c, n, ninv));
    }
}

/// src/hal/cpu.rs:983-1015 (wide == 0) and :1018-1057 (wide == 1)
__global__ void __launch_bounds__(256) bconv_pow2_kernel(KView d, KView src, i128 f0, i128 f1, int shift, int log2m,
                                                         int wide, int64_t lines, int chunks) {
    const i128 half = (i128)1 << (shift - 1);
    const u128 mask = ((u128)1 << log2m) - 1;
    const i128 modulus = (i128)1 << log2m;
    const i128 mhalf = modulus / 2;
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;  // (i, k)
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, i = line / d.n2;
        i128 v, corr;
        if (wide) {
            i128 lo = ld128(kat<longlong2>(src, i, 0, k, l)), hi = ld128(kat<longlong2>(src, i, 1, k, l));
            v = (i128)((u128)lo + ((u128)hi << 64));
            corr = ld128(kat<longlong2>(src, i, 2, k, l));
        } else {
            v = ld128(kat<longlong2>(src, i, 0, k, l));
            corr = ld128(kat<longlong2>(src, i, 1, k, l));
        }
        i128 quot = (i128)((u128)corr + (u128)half) >> shift;
        u128 x = ((u128)v - (u128)quot * (u128)f0) * (u128)f1;
        i128 red = (i128)(x & mask);
        i128 c = red > mhalf ? red - modulus : red;
        if (wide) {
            int64_t lo = (int64_t)(uint64_t)c;
            int64_t hi = (int64_t)((c - (i128)lo) >> 64);
            *kat<int64_t>(d, i, 0, k, l) = lo;
            *kat<int64_t>(d, i, 1, k, l) = hi;
        } else {
            *kat<int64_t>(d, i, 0, k, l) = (int64_t)c;
        }
    }
}

/// dst[e] = src[perm[e]] along dimension 2 or 3 (src/hal/cpu.rs:1086-1122)
__global__ void __launch_bounds__(256) permute_kernel(KView d, KView s, const uint32_t* perm, int dim, int64_t lines,
                                                      int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, r = line / d.n2;
        int64_t j = r % d.n1, i = r / d.n1;
        int64_t v = dim == 2 ? *kat<int64_t>(s, i, j, perm[k], l) : *kat<int64_t>(s, i, j, k, perm[l]);
        *kat<int64_t>(d, i, j, k, l) = v;
    }
}

/// Grid of the line kernels, or false when the line count exceeds the grid's y dimension.
bool line_grid(const KView& d, int64_t lines, dim3* grid) {
    if (lines > 65535 || d.n1 > INT32_MAX || d.n2 > INT32_MAX) return false;
    *grid = dim3((unsigned)((d.n3 + LINE_SPAN - 1) / LINE_SPAN), (unsigned)lines, 1);
    return true;
}

void grid_for(hc_context ctx, const KView& d, int64_t lines, int* chunks, unsigned* blocks) {
    *chunks = (int)((d.n3 + 255) / 256);
    int64_t tiles = lines * *chunks;
    int64_t cap = (int64_t)hc::num_sms(ctx) * 32;
    *blocks = (unsigned)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

}  // namespace

namespace hc {

hc_status launch_pointwise(hc_context ctx, int op, const KView& d, const KView& a, const KView& b, const KMods& m) {
    int64_t lines = d.n0 * d.n1 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    int chunks;
    unsigned blocks;
    grid_for(ctx, d, lines, &chunks, &blocks);
    cudaStream_t s = stream_of(ctx);
    dim3 lg;
    const bool by_line = line_grid(d, lines, &lg);
#define HC_PW(OPV)                                                      \
    case OPV:                                                           \
        if (by_line) pw_line_kernel<OPV><<<lg, 256, 0, s>>>(d, a, b, m); \
        else pw_kernel<OPV><<<blocks, 256, 0, s>>>(d, a, b, m, lines, chunks); \
        break;
    switch (op) {
        HC_PW(OP_ASSIGN)
        HC_PW(OP_ASSIGN_NARROW)
        HC_PW(OP_ASSIGN_I128)
        HC_PW(OP_ADD_I64)
        HC_PW(OP_SUB_I64)
        HC_PW(OP_ADD_I128)
        HC_PW(OP_FMA_I64)
        HC_PW(OP_MUL_I64)
        HC_PW(OP_MUL_MONT)
        HC_PW(OP_ADD_RED_DOUBLE)
        HC_PW(OP_RED_DOUBLE)
        HC_PW(OP_ADD_RED)
        HC_PW(OP_RED)
        HC_PW(OP_I128_TO_MONT)
        HC_PW(OP_I64_TO_MONT)
        default: return fail(HC_ERR_ARG, "unknown pointwise operation");
    }
#undef HC_PW
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "pointwise kernel launch");
}

hc_status launch_matmul(hc_context ctx, const KView& d, const KView& lhs, const KView& rhs, int64_t U) {
    int64_t lines = d.n0 * d.n2;
    if (lines == 0 || d.n3 == 0 || d.n1 == 0) return HC_OK;
    int chunks;
    unsigned blocks;
    grid_for(ctx, d, lines, &chunks, &blocks);
    matmul_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(d, lhs, rhs, U, lines, chunks);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "matmul kernel launch");
}

hc_status launch_inner_product(hc_context ctx, const KView& d, const KView* l, const KView* r, int n) {
    int64_t lines = d.n0 * d.n1 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    Terms t;
    for (int i = 0; i < n; i++) t.l[i] = l[i], t.r[i] = r[i];
    t.n = n;
    int chunks;
    unsigned blocks;
    dim3 lg;
    if (line_grid(d, lines, &lg)) {
        inner_product_line_kernel<<<lg, 256, 0, stream_of(ctx)>>>(d, t);
    } else {
        grid_for(ctx, d, lines, &chunks, &blocks);
        inner_product_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(d, t, lines, chunks);
    }
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "inner product kernel launch");
}

hc_status launch_bconv_correct(hc_context ctx, const KView& d, const KView& lhs, const KView& rhs, const KMods& m,
                               int shift) {
    int64_t lines = d.n0 * d.n1 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    int chunks;
    unsigned blocks;
    dim3 lg;
    if (line_grid(d, lines, &lg)) {
        bconv_correct_line_kernel<<<lg, 256, 0, stream_of(ctx)>>>(d, lhs, rhs, m, shift);
    } else {
        grid_for(ctx, d, lines, &chunks, &blocks);
        bconv_correct_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(d, lhs, rhs, m, shift, lines, chunks);
    }
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "bconv correction kernel launch");
}

hc_status launch_bconv_pow2(hc_context ctx, const KView& d, const KView& src, i128 f0, i128 f1, int shift, int log2m,
                            int wide) {
    int64_t lines = d.n0 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    int chunks;
    unsigned blocks;
    grid_for(ctx, d, lines, &chunks, &blocks);
    bconv_pow2_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(d, src, f0, f1, shift, log2m, wide, lines, chunks);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "bconv pow2 kernel launch");
}

hc_status launch_permute(hc_context ctx, const KView& d, const KView& s, const uint32_t* perm, int dim) {
    int64_t lines = d.n0 * d.n1 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    int chunks;
    unsigned blocks;
    grid_for(ctx, d, lines, &chunks, &blocks);
    permute_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(d, s, perm, dim, lines, chunks);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "permute kernel launch");
}

}  // namespace hc
