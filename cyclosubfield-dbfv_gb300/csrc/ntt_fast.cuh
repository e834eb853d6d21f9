// Specialised NTT kernels for the factorisations of the two large field descriptors:
//   dimension 3 lines   [2, 3, 8, 64] (field_36864, deg_K = 3072)  and [3, 64, 64] (field_49152, 12288)
//   dimension 2 columns [4, 3]        (field_36864, deg_L' = 12)    and [4]         (field_49152, 4)
// They execute the same stage programs as the generic kernel (same butterflies, same order, the
// same reduction/skip/fused-final decisions read from the plan), so results are bit-identical; what
// differs is the schedule:
//  * every stage geometry is a compile-time constant, so index arithmetic is shifts and
//    immediate offsets;
//  * lines: the first register pass reads its elements straight from global memory and runs the
//    leading radix-2/radix-3 factors together; the remaining radix-2 stages run three at a time on
//    eight elements per thread; the tile lives in shared memory padded by one word per eight
//    words, which keeps the strided 64-bit accesses of every pass free of bank conflicts while
//    leaving all offsets inside a group constant;
//  * columns: one thread transforms a whole column (12 or 4 residues) in registers, loading and
//    storing it coalesced across neighbouring columns - no shared memory at all;
//  * a twiddle-1 butterfly skips its multiplication only where the skip is uniform across the
//    warp (a stage with a single twiddle block); elsewhere the product is computed and the
//    unmultiplied value selected, exactly as the reference's result requires.
#pragma once

namespace fast {

/// Index of tile element i in the padded shared-memory layout.
__device__ __forceinline__ int pad8(int i) { return i + (i >> 3); }
/// Constant offset of group element m (stride `span`) from the padded group base (valid for the
/// group geometries used here: span a multiple of 8, or span < 8 with the base's low bits < span).
__host__ __device__ constexpr int goff(int m, int span) { return m * span + ((m * span) >> 3); }

struct Ctx {
    int64_t n, one_z, one_u, il_z, il_u;
    const int64_t* tw;  // staged twiddle pairs
};

__device__ __forceinline__ void twl(const Ctx& c, int idx, int64_t& z, int64_t& u) {
    const longlong2 w = reinterpret_cast<const longlong2*>(c.tw)[idx];
    z = w.x, u = w.y;
}

/// Stage flags of the program, read once per pass (uniform).
struct SF {
    int tw_off, zeta_off;
    bool red, skip_ok, last;
};

/// The plan's reduction / skip / fused-final schedule read at run time (any prime).
struct DynSched {
    const DevStage* st;
    __device__ __forceinline__ bool red(int s) const { return st[s].reduce_before; }
    __device__ __forceinline__ bool skip(int s) const { return st[s].skip_ok; }
    __device__ __forceinline__ bool last(int s) const { return st[s].last; }
};
/// A schedule known at compile time (bit s = the flag of stage s), for primes whose plan has
/// exactly this schedule; the flags then fold into straight-line code.
template <uint32_t RED, uint32_t SKIP, uint32_t LAST>
struct FixSched {
    const DevStage* st;
    __device__ __forceinline__ bool red(int s) const { return (RED >> s) & 1; }
    __device__ __forceinline__ bool skip(int s) const { return (SKIP >> s) & 1; }
    __device__ __forceinline__ bool last(int s) const { return (LAST >> s) & 1; }
};

template <class SCH>
__device__ __forceinline__ SF sflags(const SCH& sch, int s) {
    SF f;
    f.tw_off = sch.st[s].tw_off, f.zeta_off = sch.st[s].zeta_off;
    f.red = sch.red(s), f.skip_ok = sch.skip(s), f.last = sch.last(s);
    return f;
}

__device__ __forceinline__ int64_t red1(const Ctx& c, int64_t x) { return bmul1(c.one_u, x, c.n); }

// ---------------------------------------------------------------- butterflies

/// Forward radix-2 butterfly of block `tb` (src/hal/ntt.rs:338-349). UNIFORM0: the block is 0
/// for the whole warp, so a permitted skip avoids the product.
template <bool UNIFORM0>
__device__ __forceinline__ void fwd2(const Ctx& c, const SF& f, bool fuse, int tb, int64_t& x, int64_t& y) {
    int64_t t;
    if (UNIFORM0) {
        if (f.skip_ok) {
            t = y;
        } else {
            int64_t z, u;
            twl(c, f.tw_off, z, u);
            t = bmul(z, u, y, c.n);
        }
    } else {
        int64_t z, u;
        twl(c, f.tw_off + tb, z, u);
        t = bmul(z, u, y, c.n);
        if (f.skip_ok && tb == 0) t = y;
    }
    int64_t o0 = wadd(x, t), o1 = wsub(x, t);
    if (fuse) {
        o0 = red1(c, o0);
        o1 = red1(c, o1);
    }
    x = o0;
    y = o1;
}

/// Forward radix-3 butterfly of block `blk` (src/hal/ntt.rs:386-406).
template <bool UNIFORM0>
__device__ __forceinline__ void fwd3(const Ctx& c, const SF& f, bool fuse, int blk, int64_t& a, int64_t& b,
                                     int64_t& d) {
    const int base = f.tw_off + 6 * blk;
    int64_t w0z, w0u, w1z, w1u, w2z, w2u, w3z, w3u, w4z, w4u, w5z, w5u;
    twl(c, base + 1, w1z, w1u);
    twl(c, base + 2, w2z, w2u);
    twl(c, base + 4, w4z, w4u);
    twl(c, base + 5, w5z, w5u);
    int64_t t_b, t_c;
    if (UNIFORM0 && f.skip_ok) {
        t_b = b;
        t_c = d;
    } else {
        twl(c, base, w0z, w0u);
        twl(c, base + 3, w3z, w3u);
        t_b = bmul(w0z, w0u, b, c.n);
        t_c = bmul(w3z, w3u, d, c.n);
        if (!UNIFORM0 && f.skip_ok && w0z == 1) {
            t_b = b;
            t_c = d;
        }
    }
    const int64_t t_bz = bmul(w1z, w1u, b, c.n), t_bzz = bmul(w2z, w2u, b, c.n);
    const int64_t t_cz = bmul(w4z, w4u, d, c.n), t_czz = bmul(w5z, w5u, d, c.n);
    int64_t o0 = wadd(wadd(a, t_b), t_c), o1 = wadd(wadd(a, t_bz), t_czz), o2 = wadd(wadd(a, t_bzz), t_cz);
    if (fuse) {
        o0 = red1(c, o0);
        o1 = red1(c, o1);
        o2 = red1(c, o2);
    }
    a = o0;
    b = o1;
    d = o2;
}

/// Inverse radix-3 butterfly of a factor-3 stage (src/hal/ntt.rs:511-530). Every radix-3 stage
/// of the specialised shapes is the single stage of a factor of length 3: it has one block, whose
/// twiddles are v^0 = 1, so the reference's twiddle-1 skip always applies and the outputs take
/// no block-twiddle product (only the fused len^-1 scaling when the stage is the last one).
__device__ __forceinline__ void inv3(const Ctx& c, const SF& f, int64_t& a, int64_t& b, int64_t& d) {
    int64_t zz0, zu0, zz1, zu1;
    twl(c, f.zeta_off, zz0, zu0);
    twl(c, f.zeta_off + 1, zz1, zu1);
    const int64_t y1z = bmul(zz0, zu0, b, c.n), y1zz = bmul(zz1, zu1, b, c.n);
    const int64_t y2z = bmul(zz0, zu0, d, c.n), y2zz = bmul(zz1, zu1, d, c.n);
    const int64_t s0 = wadd(wadd(a, b), d);
    const int64_t sy = wadd(wadd(a, y1zz), y2z), sz = wadd(wadd(a, y1z), y2zz);
    if (f.last) {
        a = bmul(c.il_z, c.il_u, s0, c.n);
        b = bmul(c.il_z, c.il_u, sy, c.n);
        d = bmul(c.il_z, c.il_u, sz, c.n);
        return;
    }
    a = s0;
    b = sy;
    d = sz;
}

// ---------------------------------------------------------------- register groups of radix-2 stages

/// K forward radix-2 stages on the group x[0..2^K) (element m at distance m * span). block0:
/// the group's twiddle block at the first stage (0 for the whole warp when NB0 == 1).
template <int K, bool NB1>
__device__ __forceinline__ void fwd_group(const Ctx& c, const SF* f, const bool* fuse, int block0, int64_t* x) {
    constexpr int M = 1 << K;
#pragma unroll
    for (int q = 0; q < K; q++) {
        if (f[q].red) {
#pragma unroll
            for (int m = 0; m < M; m++) x[m] = red1(c, x[m]);
        }
        const int half = M >> (q + 1);
#pragma unroll
        for (int j = 0; j < M / 2; j++) {
            const int m1 = ((j / half) * 2 * half) + (j % half), m2 = m1 + half;
            const int tbc = m1 >> (K - q);  // compile-time part of the block
            if (NB1 && tbc == 0) fwd2<true>(c, f[q], fuse[q], 0, x[m1], x[m2]);
            else fwd2<false>(c, f[q], fuse[q], (block0 << q) + tbc, x[m1], x[m2]);
        }
    }
}

/// K inverse radix-2 stages (distances growing) on the group x[0..2^K); blockK: the group's block
/// at the pass's last stage (NBK1: 0 for the whole warp).
template <int K, bool NBK1>
__device__ __forceinline__ void inv_group(const Ctx& c, const SF* f, int blockK, int64_t* x) {
    constexpr int M = 1 << K;
#pragma unroll
    for (int q = 0; q < K; q++) {
        if (f[q].red) {
#pragma unroll
            for (int m = 0; m < M; m++) x[m] = red1(c, x[m]);
        }
        const int dist = 1 << q;
#pragma unroll
        for (int j = 0; j < M / 2; j++) {
            const int m1 = ((j >> q) << (q + 1)) | (j & (dist - 1)), m2 = m1 + dist;
            const int tbc = m1 >> (q + 1);
            const int64_t sum = wadd(x[m1], x[m2]), dif = wsub(x[m1], x[m2]);
            if (f[q].last) {
                x[m1] = bmul(c.il_z, c.il_u, sum, c.n);
                x[m2] = bmul(c.il_z, c.il_u, dif, c.n);
            } else if (NBK1 && tbc == 0) {
                // block 0 for the whole warp: twiddle 1, product skipped
                x[m1] = sum;
                x[m2] = dif;
            } else {
                const int tb = (blockK << (K - 1 - q)) + tbc;
                int64_t z, u;
                twl(c, f[q].tw_off + tb, z, u);
                int64_t t = bmul(z, u, dif, c.n);
                if (z == 1) t = dif;
                x[m1] = sum;
                x[m2] = t;
            }
        }
    }
}

/// One pass of K radix-2 stages of a factor over a padded shared-memory tile: groups of 2^K
/// elements at distance SPAN (= 2^LOG_SPAN) inside blocks of 2^LOG_GLEN elements, 2^LOG_NB twiddle
/// blocks per factor at the pass's reference stage (first stage forward, last stage inverse).
template <bool INV, int K, int LOG_SPAN, int LOG_GLEN, int LOG_NB, class SCH>
__device__ __forceinline__ void r2_pass(const Ctx& c, int64_t* s, int ngroups, const SCH& sch, int s0,
                                        bool reduce_output) {
    constexpr int M = 1 << K, SPAN = 1 << LOG_SPAN;
    SF f[K];
    bool fuse[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        f[q] = sflags(sch, s0 + q);
        fuse[q] = f[q].last && reduce_output;
    }
    for (int gg = threadIdx.x; gg < ngroups; gg += blockDim.x) {
        const int g = gg >> LOG_SPAN, o = gg & (SPAN - 1);
        const int blk = g & ((1 << LOG_NB) - 1);
        const int base = (g << LOG_GLEN) + o;
        int64_t* p = s + pad8(base);
        int64_t x[M];
#pragma unroll
        for (int m = 0; m < M; m++) x[m] = p[goff(m, SPAN)];
        if (INV) inv_group<K, LOG_NB == 0>(c, f, blk, x);
        else fwd_group<K, LOG_NB == 0>(c, f, fuse, blk, x);
#pragma unroll
        for (int m = 0; m < M; m++) p[goff(m, SPAN)] = x[m];
    }
}

// ---------------------------------------------------------------- lines

/// Copies a padded tile of `len` elements to global memory, multiplying (mode 2/3) by
/// mulp[e * me] in Montgomery form.
__device__ __forceinline__ void line_store(const int64_t* s, int64_t* g, int len, bool mul, const int64_t* mulp,
                                           int64_t me, int64_t mn, int64_t mi) {
    for (int e = threadIdx.x; e < len; e += blockDim.x) {
        int64_t v = s[pad8(e)];
        if (mul) v = mul_mont(v, mulp[e * me], mn, mi);
        g[e] = v;
    }
}

/// Reduces every element of a register group when the stage asks for it (src/hal/ntt.rs: the
/// reduction pass before a stage whose growth could overflow).
template <int N>
__device__ __forceinline__ void red_all(const Ctx& c, bool red, int64_t* x) {
    if (red) {
#pragma unroll
        for (int m = 0; m < N; m++) x[m] = red1(c, x[m]);
    }
}

/// [2, 3, 8, 64] line (3072 residues): g -> g, via the padded tile s (3456 words). MODE as the
/// tile kernel (0 forward, 1 inverse, 2 forward + product, 3 inverse + product); the schedule
/// SCH is that of the programme of MODE's direction. Stages: 0 = factor 2, 1 = factor 3,
/// 2..4 = factor 8, 5..10 = factor 64.
template <int MODE, class SCH>
__device__ __forceinline__ void line3072(const SCH& sch, const Ctx& c, int64_t* s, int64_t* g, const int64_t* mulp,
                                         int64_t me, int64_t mn, int64_t mi) {
    constexpr bool inv = MODE & 1, reduce_output = MODE == 0;
    // pass 1: factors 2 (distance 1536) and 3 (distance 512), straight from global memory
    {
        const SF f0 = sflags(sch, 0), f1 = sflags(sch, 1);
        const bool fz0 = f0.last && reduce_output, fz1 = f1.last && reduce_output;
        for (int o = threadIdx.x; o < 512; o += blockDim.x) {
            int64_t x[2][3];
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int a = 0; a < 3; a++) x[b][a] = g[o + 512 * a + 1536 * b];
            red_all<6>(c, f0.red, &x[0][0]);
            if (!inv) {
#pragma unroll
                for (int a = 0; a < 3; a++) fwd2<true>(c, f0, fz0, 0, x[0][a], x[1][a]);
                red_all<6>(c, f1.red, &x[0][0]);
#pragma unroll
                for (int b = 0; b < 2; b++) fwd3<true>(c, f1, fz1, 0, x[b][0], x[b][1], x[b][2]);
            } else {
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    // factor 2: one block, twiddle 1 unless fused
                    const int64_t sum = wadd(x[0][a], x[1][a]), dif = wsub(x[0][a], x[1][a]);
                    if (f0.last) {
                        x[0][a] = bmul(c.il_z, c.il_u, sum, c.n);
                        x[1][a] = bmul(c.il_z, c.il_u, dif, c.n);
                    } else {
                        x[0][a] = sum;
                        x[1][a] = dif;
                    }
                }
                red_all<6>(c, f1.red, &x[0][0]);
#pragma unroll
                for (int b = 0; b < 2; b++) inv3(c, f1, x[b][0], x[b][1], x[b][2]);
            }
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int a = 0; a < 3; a++) s[pad8(o + 512 * a + 1536 * b)] = x[b][a];
        }
    }
    __syncthreads();
    if (!inv) {
        r2_pass<false, 3, 6, 9, 0>(c, s, 384, sch, 2, reduce_output);  // factor 8: distances 256, 128, 64
        __syncthreads();
        r2_pass<false, 3, 3, 6, 0>(c, s, 384, sch, 5, reduce_output);  // factor 64: 32, 16, 8
        __syncthreads();
        r2_pass<false, 3, 0, 3, 3>(c, s, 384, sch, 8, reduce_output);  // factor 64: 4, 2, 1
    } else {
        r2_pass<true, 3, 6, 9, 0>(c, s, 384, sch, 2, false);  // factor 8: distances 64, 128, 256
        __syncthreads();
        r2_pass<true, 3, 0, 3, 3>(c, s, 384, sch, 5, false);  // factor 64: 1, 2, 4
        __syncthreads();
        r2_pass<true, 3, 3, 6, 0>(c, s, 384, sch, 8, false);  // factor 64: 8, 16, 32
    }
    __syncthreads();
    line_store(s, g, 3072, MODE & 2, mulp, me, mn, mi);
}

/// [3, 64, 64] line (12288 residues): stages 0 = factor 3 (distance 4096), 1..6 = first factor
/// 64 (distances 2048 .. 64), 7..12 = second factor 64 (32 .. 1).
template <int MODE, class SCH>
__device__ __forceinline__ void line12288(const SCH& sch, const Ctx& c, int64_t* s, int64_t* g, const int64_t* mulp,
                                          int64_t me, int64_t mn, int64_t mi) {
    constexpr bool inv = MODE & 1, reduce_output = MODE == 0;
    // pass 1: factor 3 and three stages of the first factor 64, straight from global memory
    {
        SF f[4];
        bool fz[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            f[q] = sflags(sch, q);
            fz[q] = f[q].last && reduce_output;
        }
        // forward: elements o + 512 m + 4096 a (o < 512); inverse: base + 64 m + 4096 a with
        // base = (gg >> 6) * 512 + (gg & 63)
        constexpr int span = inv ? 64 : 512;
        for (int gg = threadIdx.x; gg < 512; gg += blockDim.x) {
            const int base = inv ? ((gg >> 6) << 9) + (gg & 63) : gg;
            int64_t x[3][8];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int m = 0; m < 8; m++) x[a][m] = g[base + span * m + 4096 * a];
            red_all<24>(c, f[0].red, &x[0][0]);
            if (!inv) {
#pragma unroll
                for (int m = 0; m < 8; m++) fwd3<true>(c, f[0], fz[0], 0, x[0][m], x[1][m], x[2][m]);
#pragma unroll
                for (int a = 0; a < 3; a++) fwd_group<3, true>(c, f + 1, fz + 1, 0, x[a]);
            } else {
#pragma unroll
                for (int m = 0; m < 8; m++) inv3(c, f[0], x[0][m], x[1][m], x[2][m]);
#pragma unroll
                for (int a = 0; a < 3; a++) inv_group<3, false>(c, f + 1, gg >> 6, x[a]);
            }
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int m = 0; m < 8; m++) s[pad8(base + span * m + 4096 * a)] = x[a][m];
        }
    }
    __syncthreads();
    if (!inv) {
        r2_pass<false, 3, 6, 9, 3>(c, s, 1536, sch, 4, reduce_output);   // factor 64 (a): 256, 128, 64
        __syncthreads();
        r2_pass<false, 3, 3, 6, 0>(c, s, 1536, sch, 7, reduce_output);   // factor 64 (b): 32, 16, 8
        __syncthreads();
        r2_pass<false, 3, 0, 3, 3>(c, s, 1536, sch, 10, reduce_output);  // factor 64 (b): 4, 2, 1
    } else {
        r2_pass<true, 3, 9, 12, 0>(c, s, 1536, sch, 4, false);  // factor 64 (a): 512, 1024, 2048
        __syncthreads();
        r2_pass<true, 3, 0, 3, 3>(c, s, 1536, sch, 7, false);   // factor 64 (b): 1, 2, 4
        __syncthreads();
        r2_pass<true, 3, 3, 6, 0>(c, s, 1536, sch, 10, false);  // factor 64 (b): 8, 16, 32
    }
    __syncthreads();
    line_store(s, g, 12288, MODE & 2, mulp, me, mn, mi);
}

/// One of the three 4096-residue blocks of a [3, 64, 64] line, computed by one CTA of a 3-CTA
/// cluster: the factor-3 stage couples the blocks, but each output of a radix-3 butterfly needs
/// only its own two twiddle products, so the CTA of block `blk` reads all three inputs of its
/// positions and computes just its output; the remaining 12 stages act within the block. The
/// line is transformed in place, so no CTA may store before all three have read their inputs:
/// `cluster_sync` (a cluster-wide barrier) separates the first pass from the stores.
template <int MODE, class SCH, class SYNC>
__device__ __forceinline__ void line12288_block(const SCH& sch, const Ctx& c, int64_t* s, int64_t* g, int blk,
                                                const int64_t* mulp, int64_t me, int64_t mn, int64_t mi,
                                                SYNC cluster_sync) {
    constexpr bool inv = MODE & 1, reduce_output = MODE == 0;
    {
        SF f[4];
        bool fz[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            f[q] = sflags(sch, q);
            fz[q] = f[q].last && reduce_output;
        }
        // twiddles of the factor-3 stage (one block, whose block twiddles are 1: the inverse
        // outputs take no block-twiddle product, as inv3 explains)
        int64_t wz0, wu0, wz1, wu1;  // forward: the two products of output blk; inverse: zeta, zeta^2
        if (!inv) {
            const int i0 = blk == 0 ? 0 : (blk == 1 ? 1 : 2), i1 = blk == 0 ? 3 : (blk == 1 ? 5 : 4);
            twl(c, f[0].tw_off + i0, wz0, wu0);
            twl(c, f[0].tw_off + i1, wz1, wu1);
        } else {
            twl(c, f[0].zeta_off, wz0, wu0);
            twl(c, f[0].zeta_off + 1, wz1, wu1);
        }
        constexpr int span = inv ? 64 : 512;
        for (int gg = threadIdx.x; gg < 512; gg += blockDim.x) {
            const int base = inv ? ((gg >> 6) << 9) + (gg & 63) : gg;
            int64_t x[8];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int p = base + span * m;
                int64_t a = g[p], b = g[p + 4096], d = g[p + 8192];
                if (f[0].red) {
                    a = red1(c, a);
                    b = red1(c, b);
                    d = red1(c, d);
                }
                int64_t o;
                if (!inv) {
                    // src/hal/ntt.rs:386-406, output blk of the butterfly
                    int64_t tb, tc;
                    if (blk == 0 && f[0].skip_ok) {
                        tb = b;
                        tc = d;
                    } else {
                        tb = bmul(wz0, wu0, b, c.n);
                        tc = bmul(wz1, wu1, d, c.n);
                    }
                    o = wadd(wadd(a, tb), tc);
                    if (fz[0]) o = red1(c, o);
                } else {
                    // src/hal/ntt.rs:511-530, output blk of the butterfly
                    if (blk == 0) {
                        o = wadd(wadd(a, b), d);
                    } else if (blk == 1) {
                        o = wadd(wadd(a, bmul(wz1, wu1, b, c.n)), bmul(wz0, wu0, d, c.n));
                    } else {
                        o = wadd(wadd(a, bmul(wz0, wu0, b, c.n)), bmul(wz1, wu1, d, c.n));
                    }
                    if (f[0].last) o = bmul(c.il_z, c.il_u, o, c.n);
                }
                x[m] = o;
            }
            if (!inv) fwd_group<3, true>(c, f + 1, fz + 1, 0, x);
            else inv_group<3, false>(c, f + 1, gg >> 6, x);
#pragma unroll
            for (int m = 0; m < 8; m++) s[pad8(base + span * m)] = x[m];
        }
    }
    cluster_sync();  // also a barrier of this CTA
    if (!inv) {
        r2_pass<false, 3, 6, 9, 3>(c, s, 512, sch, 4, reduce_output);   // factor 64 (a): 256, 128, 64
        __syncthreads();
        r2_pass<false, 3, 3, 6, 0>(c, s, 512, sch, 7, reduce_output);   // factor 64 (b): 32, 16, 8
        __syncthreads();
        r2_pass<false, 3, 0, 3, 3>(c, s, 512, sch, 10, reduce_output);  // factor 64 (b): 4, 2, 1
    } else {
        r2_pass<true, 3, 9, 12, 0>(c, s, 512, sch, 4, false);  // factor 64 (a): 512, 1024, 2048
        __syncthreads();
        r2_pass<true, 3, 0, 3, 3>(c, s, 512, sch, 7, false);   // factor 64 (b): 1, 2, 4
        __syncthreads();
        r2_pass<true, 3, 3, 6, 0>(c, s, 512, sch, 10, false);  // factor 64 (b): 8, 16, 32
    }
    __syncthreads();
    line_store(s, g + 4096 * blk, 4096, MODE & 2, mulp + (me ? 4096 * blk : 0), me, mn, mi);
}

/// A [3, 64, 64] line with a tile of one 4096-residue block (for kernels that cannot give a CTA the
/// whole 12288-residue line): stage 0, the factor-3 stage that couples the three blocks, runs in
/// place in global memory, each thread owning whole position triples (the butterfly of line12288's
/// first pass); stages 1..12, which act within a block, then run block by block exactly as
/// line12288_block runs them. The first pass's global writes are the CTA's own, visible to its
/// threads after the barrier.
template <int MODE, class SCH>
__device__ __forceinline__ void line12288_seq(const SCH& sch, const Ctx& c, int64_t* s, int64_t* g,
                                              const int64_t* mulp, int64_t me, int64_t mn, int64_t mi) {
    constexpr bool inv = MODE & 1, reduce_output = MODE == 0;
    SF f[4];
    bool fz[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        f[q] = sflags(sch, q);
        fz[q] = f[q].last && reduce_output;
    }
    for (int p = threadIdx.x; p < 4096; p += blockDim.x) {
        int64_t a = g[p], b = g[p + 4096], d = g[p + 8192];
        if (f[0].red) {
            a = red1(c, a);
            b = red1(c, b);
            d = red1(c, d);
        }
        if (!inv) fwd3<true>(c, f[0], fz[0], 0, a, b, d);
        else inv3(c, f[0], a, b, d);
        g[p] = a, g[p + 4096] = b, g[p + 8192] = d;
    }
    __syncthreads();
    constexpr int span = inv ? 64 : 512;
    for (int blk = 0; blk < 3; blk++) {
        int64_t* gb = g + 4096 * blk;
        for (int gg = threadIdx.x; gg < 512; gg += blockDim.x) {
            const int base = inv ? ((gg >> 6) << 9) + (gg & 63) : gg;
            int64_t x[8];
#pragma unroll
            for (int m = 0; m < 8; m++) x[m] = gb[base + span * m];
            if (!inv) fwd_group<3, true>(c, f + 1, fz + 1, 0, x);
            else inv_group<3, false>(c, f + 1, gg >> 6, x);
#pragma unroll
            for (int m = 0; m < 8; m++) s[pad8(base + span * m)] = x[m];
        }
        __syncthreads();
        if (!inv) {
            r2_pass<false, 3, 6, 9, 3>(c, s, 512, sch, 4, reduce_output);   // factor 64 (a): 256, 128, 64
            __syncthreads();
            r2_pass<false, 3, 3, 6, 0>(c, s, 512, sch, 7, reduce_output);   // factor 64 (b): 32, 16, 8
            __syncthreads();
            r2_pass<false, 3, 0, 3, 3>(c, s, 512, sch, 10, reduce_output);  // factor 64 (b): 4, 2, 1
        } else {
            r2_pass<true, 3, 9, 12, 0>(c, s, 512, sch, 4, false);  // factor 64 (a): 512, 1024, 2048
            __syncthreads();
            r2_pass<true, 3, 0, 3, 3>(c, s, 512, sch, 7, false);   // factor 64 (b): 1, 2, 4
            __syncthreads();
            r2_pass<true, 3, 3, 6, 0>(c, s, 512, sch, 10, false);  // factor 64 (b): 8, 16, 32
        }
        __syncthreads();
        line_store(s, gb, 4096, MODE & 2, mulp + (me ? 4096 * blk : 0), me, mn, mi);
        __syncthreads();  // the tile is refilled by the next block
    }
}

// ---------------------------------------------------------------- columns

/// [4, 3] column (12 residues at element stride ge): factor 4 (distance 3) then factor 3
/// (distance 1). Forward stages: 0 = factor 4 length 4, 1 = factor 4 length 2, 2 = factor 3;
/// inverse stages: 0 = factor 4 length 2, 1 = factor 4 length 4, 2 = factor 3.
__device__ __forceinline__ void col12(const Ctx& c, const SF* f, bool inv, bool reduce_output, int64_t (&x)[4][3]) {
    if (!inv) {
        if (f[0].red)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = red1(c, x[a][b]);
        const bool z0 = f[0].last && reduce_output, z1 = f[1].last && reduce_output, z2 = f[2].last && reduce_output;
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) fwd2<true>(c, f[0], z0, 0, x[a][b], x[a + 2][b]);
        if (f[1].red)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = red1(c, x[a][b]);
#pragma unroll
        for (int b = 0; b < 3; b++) {
            fwd2<true>(c, f[1], z1, 0, x[0][b], x[1][b]);
            // block 1: an ordinary twiddle (not 1), product always taken
            int64_t z, u;
            twl(c, f[1].tw_off + 1, z, u);
            const int64_t t = bmul(z, u, x[3][b], c.n);
            int64_t o0 = wadd(x[2][b], t), o1 = wsub(x[2][b], t);
            if (z1) {
                o0 = red1(c, o0);
                o1 = red1(c, o1);
            }
            x[2][b] = o0;
            x[3][b] = o1;
        }
        if (f[2].red)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = red1(c, x[a][b]);
#pragma unroll
        for (int a = 0; a < 4; a++) fwd3<true>(c, f[2], z2, 0, x[a][0], x[a][1], x[a][2]);
    } else {
        if (f[0].red)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = red1(c, x[a][b]);
#pragma unroll
        for (int b = 0; b < 3; b++) {
            // factor 4, length-2 stage: block 0 (pair 0, 1) and block 1 (pair 2, 3)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int64_t sum = wadd(x[2 * h][b], x[2 * h + 1][b]), dif = wsub(x[2 * h][b], x[2 * h + 1][b]);
                if (f[0].last) {
                    x[2 * h][b] = bmul(c.il_z, c.il_u, sum, c.n);
                    x[2 * h + 1][b] = bmul(c.il_z, c.il_u, dif, c.n);
                } else if (h == 0) {
                    x[0][b] = sum;
                    x[1][b] = dif;
                } else {
                    int64_t z, u;
                    twl(c, f[0].tw_off + 1, z, u);
                    int64_t t = bmul(z, u, dif, c.n);
                    if (z == 1) t = dif;
                    x[2][b] = sum;
                    x[3][b] = t;
                }
            }
        }
        if (f[1].red)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = red1(c, x[a][b]);
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                const int64_t sum = wadd(x[a][b], x[a + 2][b]), dif = wsub(x[a][b], x[a + 2][b]);
                if (f[1].last) {
                    x[a][b] = bmul(c.il_z, c.il_u, sum, c.n);
                    x[a + 2][b] = bmul(c.il_z, c.il_u, dif, c.n);
                } else {
                    x[a][b] = sum;
                    x[a + 2][b] = dif;
                }
            }
        if (f[2].red)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = red1(c, x[a][b]);
#pragma unroll
        for (int a = 0; a < 4; a++) inv3(c, f[2], x[a][0], x[a][1], x[a][2]);
    }
}

/// [4] column (4 residues): forward stages 0 = length 4, 1 = length 2; inverse the reverse.
__device__ __forceinline__ void col4(const Ctx& c, const SF* f, bool inv, bool reduce_output, int64_t (&x)[4]) {
    if (!inv) {
        if (f[0].red)
#pragma unroll
            for (int a = 0; a < 4; a++) x[a] = red1(c, x[a]);
        const bool z0 = f[0].last && reduce_output, z1 = f[1].last && reduce_output;
        fwd2<true>(c, f[0], z0, 0, x[0], x[2]);
        fwd2<true>(c, f[0], z0, 0, x[1], x[3]);
        if (f[1].red)
#pragma unroll
            for (int a = 0; a < 4; a++) x[a] = red1(c, x[a]);
        fwd2<true>(c, f[1], z1, 0, x[0], x[1]);
        int64_t z, u;
        twl(c, f[1].tw_off + 1, z, u);
        const int64_t t = bmul(z, u, x[3], c.n);
        int64_t o0 = wadd(x[2], t), o1 = wsub(x[2], t);
        if (z1) {
            o0 = red1(c, o0);
            o1 = red1(c, o1);
        }
        x[2] = o0;
        x[3] = o1;
    } else {
        if (f[0].red)
#pragma unroll
            for (int a = 0; a < 4; a++) x[a] = red1(c, x[a]);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int64_t sum = wadd(x[2 * h], x[2 * h + 1]), dif = wsub(x[2 * h], x[2 * h + 1]);
            if (f[0].last) {
                x[2 * h] = bmul(c.il_z, c.il_u, sum, c.n);
                x[2 * h + 1] = bmul(c.il_z, c.il_u, dif, c.n);
            } else if (h == 0) {
                x[0] = sum;
                x[1] = dif;
            } else {
                int64_t z, u;
                twl(c, f[0].tw_off + 1, z, u);
                int64_t t = bmul(z, u, dif, c.n);
                if (z == 1) t = dif;
                x[2] = sum;
                x[3] = t;
            }
        }
        if (f[1].red)
#pragma unroll
            for (int a = 0; a < 4; a++) x[a] = red1(c, x[a]);
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const int64_t sum = wadd(x[a], x[a + 2]), dif = wsub(x[a], x[a + 2]);
            if (f[1].last) {
                x[a] = bmul(c.il_z, c.il_u, sum, c.n);
                x[a + 2] = bmul(c.il_z, c.il_u, dif, c.n);
            } else {
                x[a] = sum;
                x[a + 2] = dif;
            }
        }
    }
}

}  // namespace fast
