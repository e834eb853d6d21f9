// Fused ring-level kernels. Each replaces a sequence of Backend calls of the reference's ring /
// BFV layer with one pass over the data, computing exactly the same integers:
//  - bconv_fused_kernel: BEHZ base conversion, plain (BConvCache::bconv,
//    cyclosubfield-dbfv/src/ring.rs:1663-1701) and gadget-batched (GadgetBConvCache::bconv,
//    src/ring.rs:1809-1851): mul_mont64 by (q/p)^-1, the small-K matmul (exact, in 29-bit limbs),
//    the double reduction, the q~-scaled correction and the conversion to Montgomery form, without
//    the i128 `tmp` / `correction` tensors ever reaching HBM.
//  - galois_kernel: both permutation passes of apply_galois (src/ring.rs:1212-1222) as one gather.
//  - keyswitch_async_kernel (keyswitch1_kernel for odd or unaligned views): the key-switch inner
//    product, the addition of c0 / c1 through mont(1) and reduce_wide (src/bfv.rs:498-556,
//    src/ring.rs:460-485, :503-509, :846-865).
//  - tensor_kernel: hom_mul_raw_acc + reduce_wide (src/bfv.rs:667-683).
//  - giant_kernel: one giant step of the homomorphic CRT transform for up to four output digits:
//    the baby-step inner product over the digit convolution (dbfv_acc_inner_product_element_lprime,
//    src/dbfv.rs:291-399), the addition of the carried result (dbfv_acc_add, :153-163) and the
//    reduction (dbfv_finish_accumulator, :401-404), without the wide accumulator in HBM.
#include <algorithm>

#include "common.cuh"

namespace {

constexpr int BCONV_THREADS = 128;

struct BconvArgs {
    KView src;  // [ns, r, dl, dk]
    KView dst;  // [ns * nb, rd, dl, dk]
    BconvConsts c;
    int r, rd, nb;
    int ochunk;  // outputs per CTA (even): blockIdx.z selects the outputs [z ochunk, (z + 1) ochunk)
    int64_t npos;
    const int64_t* sub_mul;  // optional [2][rd]: store mul_mont(dst - v, b_j) instead of v (b_j, b_j ninv)
};

constexpr int LIMB_BITS = 29;
constexpr int LIMB_GROUP = 16;  // terms per int64 partial-sum group

/// hi:lo += a00 + a01 2^29 + a11 2^58 (a00 >= 0).
__device__ __forceinline__ void fold_limbs(uint64_t& lo, int64_t& hi, int64_t a00, int64_t a01, int64_t a11) {
    const u128 s = (u128)lo + (uint64_t)a00 + ((uint64_t)a01 << LIMB_BITS) + ((uint64_t)a11 << (2 * LIMB_BITS));
    lo = (uint64_t)s;
    hi = (int64_t)((uint64_t)hi + (uint64_t)(a01 >> (64 - LIMB_BITS)) + (uint64_t)(a11 >> (64 - 2 * LIMB_BITS)) +
                   (uint64_t)(s >> 64));
}

/// One output pair's multiply-accumulate over the lifts u in [lo, hi): the exact sums
/// sum_u m_u x_u as 128-bit words. Operands are split as v = v1 2^29 + v0 with 0 <= v0 < 2^29;
/// with |x| < 2^57 and |m| < 2^56 (so |x1| <= 2^28, |m1| <= 2^27) the products x0 m0 < 2^58,
/// |x1 m1| <= 2^55 and |(x0 + x1)(m0 + m1)| < 2^58.91 add up over 16 terms in int64 without
/// overflow; the middle column x0 m1 + x1 m0 is the Karatsuba difference of the three sums.
/// Terms [u, u + n) of one group into the six int64 column sums (xp, p0, p1 at term u).
template <int N>
__device__ __forceinline__ void limb_terms(const int2* __restrict__ xp, const int4* __restrict__ p0,
                                           const int4* __restrict__ p1, int n, int64_t (&s)[6]) {
#pragma unroll
    for (int t = 0; t < N; t++) {
        if (N == LIMB_GROUP || t < n) {
            const int2 x = xp[t * BCONV_THREADS];
            const int xs = x.x + x.y;
            const int4 p = __ldg(p0 + t), q = __ldg(p1 + t);
            s[0] += (int64_t)x.x * p.x;
            s[1] += (int64_t)x.y * p.y;
            s[2] += (int64_t)xs * p.z;
            s[3] += (int64_t)x.x * q.x;
            s[4] += (int64_t)x.y * q.y;
            s[5] += (int64_t)xs * q.z;
        }
    }
}

__device__ __forceinline__ void limb_mac2(const int2* __restrict__ xcol, const int4* __restrict__ m0,
                                          const int4* __restrict__ m1, int lo, int hi, uint64_t& l0, int64_t& h0,
                                          uint64_t& l1, int64_t& h1) {
    for (int g0 = lo; g0 < hi; g0 += LIMB_GROUP) {
        const int n = min(LIMB_GROUP, hi - g0);
        int64_t s[6] = {0, 0, 0, 0, 0, 0};  // a00, a11, am, b00, b11, bm
        const int2* xp = xcol + g0 * BCONV_THREADS;
        // a full group fully unrolled (every address an immediate offset), a partial one in
        // steps of four
        if (n == LIMB_GROUP) {
            limb_terms<LIMB_GROUP>(xp, m0 + g0, m1 + g0, n, s);
        } else {
            for (int t = 0; t < n; t += 4) limb_terms<4>(xp + t * BCONV_THREADS, m0 + g0 + t, m1 + g0 + t, n - t, s);
        }
        fold_limbs(l0, h0, s[0], s[2] - s[0] - s[1], s[1]);
        fold_limbs(l1, h1, s[3], s[5] - s[3] - s[4], s[4]);
    }
}

/// The conversion's epilogue for output j of block b: v (the double-reduced sums) plus the
/// correction mul_mont(q, qmodp), to Montgomery form, optionally dst <- mul_mont(dst - y, b_j).
template <bool SUB>
__device__ __forceinline__ void bconv_store(const BconvArgs& a, const KMods& dm, int b, int j, int64_t q, int64_t v,
                                            int64_t* p, int64_t old) {
    const int64_t n = dm.n[j], ninv = dm.ninv[j];
    const int64_t* qt = a.c.qtab + (b * a.rd + j) * (2 * a.c.qhalf + 1) + a.c.qhalf;
    const int64_t qm = (q >= -a.c.qhalf && q <= a.c.qhalf) ? __ldg(qt + q)
                                                            : mul_mont(q, a.c.qmodp[b * a.rd + j], n, ninv);
    const int64_t y = mul_mont_c(wadd(v, qm), dm.r2[j], __ldg(a.c.r2p + j), n);  // to_mont64
    if constexpr (SUB)
        *p = mul_mont_c(wsub(old, y), __ldg(a.sub_mul + j), __ldg(a.sub_mul + a.rd + j), n);
    else
        *p = y;
}

/// BEHZ base conversion of one position per thread (BConvCache::bconv, src/ring.rs:1660-1702,
/// and the gadget form of :1800-1852). CTA (x, y, z): 128 positions of source row y / nb, output
/// block y % nb (a gadget digit), outputs [z ochunk, (z + 1) ochunk) of the block; only the
/// block's own source columns are lifted. The products with the conversion matrix use its limb
/// form: the shared array holds each lift as its limb pair (x mod 2^29, x >> 29).
/// ONE_CHUNK: the block's columns form one chunk of the reference's chunked matmul (always for
/// 57-bit primes); SUB: rescale's subtract-and-multiply store (BconvArgs::sub_mul).
template <bool ONE_CHUNK, bool SUB>
__global__ void __launch_bounds__(BCONV_THREADS) bconv_fused_kernel(BconvArgs a, KMods sm, KMods dm) {
    extern __shared__ int2 xs[];  // [r][BCONV_THREADS]
    const int b = (int)(blockIdx.y % (unsigned)a.nb);
    const int64_t i = blockIdx.y / (unsigned)a.nb;
    const int jbeg = (int)blockIdx.z * a.ochunk, jend = min(a.rd, jbeg + a.ochunk);
    const int u0 = a.c.ucol[2 * b], u1 = a.c.ucol[2 * b + 1];
    const int64_t pos = (int64_t)blockIdx.x * BCONV_THREADS + threadIdx.x;
    if (pos >= a.npos) return;
    const int64_t k = pos / a.src.n3, l = pos - k * a.src.n3;
    const int64_t* __restrict__ srcp = kat<int64_t>(a.src, i, 0, k, l);       // row u at u * src.s1
    int64_t* __restrict__ dstp = kat<int64_t>(a.dst, i * a.nb + b, 0, k, l);  // row j at j * dst.s1
    // the source is multiplied by (Q/p)^-1 in Montgomery form, giving plain lifts in (-p, p)
    for (int u = u0; u < u1; u++) {
        int64_t x = srcp[u * a.src.s1];
        x = mul_mont_c(x, __ldg(a.c.qinv + u), __ldg(a.c.qinvp + u), sm.n[u]);
        xs[u * BCONV_THREADS + threadIdx.x] = make_int2((int)(x & ((1 << LIMB_BITS) - 1)), (int)(x >> LIMB_BITS));
    }
    const i128 half = (i128)1 << (a.c.shift - 1);
    const int2* xcol = xs + threadIdx.x;  // this thread's lifts, stride BCONV_THREADS
    const int64_t* __restrict__ mq = a.c.mat + ((int64_t)b * (a.rd + 1) + a.rd) * a.r;
    // the correction q = round(sum_u x_u round(2^shift / p_u) / 2^shift)
    i128 corr;
    if (a.c.corr_limb) {
        int64_t c0 = 0, c1 = 0;
#pragma unroll 4
        for (int u = u0; u < u1; u++) {
            const int2 x = xcol[u * BCONV_THREADS];
            const int m = (int)__ldg(mq + u);
            c0 += (int64_t)x.x * m;
            c1 += (int64_t)x.y * m;
        }
        corr = (i128)c0 + (i128)((u128)(i128)c1 << LIMB_BITS);
    } else {
        corr = 0;
        for (int u = u0; u < u1; u++) {
            const int2 x = xcol[u * BCONV_THREADS];
            const int64_t lift = (int64_t)x.y * ((int64_t)1 << LIMB_BITS) + x.x;
            corr = (i128)((u128)corr + (u128)((i128)__ldg(mq + u) * (i128)lift));
        }
    }
    const int64_t q = (int64_t)((i128)((u128)corr + (u128)half) >> a.c.shift);
    // two output rows per pass over the lifts (each lift is read once for both); the
    // reference's chunked matmul (src/ring.rs:1678-1691) splits the columns into chunks of
    // `chunk` (one chunk whenever r <= chunk, which holds for all 57-bit bases up to 8192
    // factors) and double-reduces each chunk's sum
    for (int j = jbeg; j < jend; j += 2) {
        const bool two = j + 1 < jend;
        const int4* __restrict__ m0 = a.c.mat3 + ((int64_t)b * a.rd + j) * a.r;
        const int4* __restrict__ m1 = two ? m0 + a.r : m0;
        int64_t v0 = 0, v1 = 0;
        // the subtract-and-multiply store's operands, loaded before the sums so that their
        // latency hides behind the multiply-accumulate
        int64_t old0 = 0, old1 = 0;
        if constexpr (SUB) {
            old0 = dstp[j * a.dst.s1];
            if (two) old1 = dstp[(j + 1) * a.dst.s1];
        }
        if constexpr (ONE_CHUNK) {
            uint64_t l0 = 0, l1 = 0;
            int64_t h0 = 0, h1 = 0;
            limb_mac2(xcol, m0, m1, u0, u1, l0, h0, l1, h1);
            v0 = double_red_words(l0, h0, dm.n[j], dm.ninv[j]);
            v1 = double_red_words(l1, h1, dm.n[j + two], dm.ninv[j + two]);
        } else {
            bool first = true;
            for (int c0 = 0; c0 < a.r; c0 += a.c.chunk) {
                const int lo = max(c0, u0), hi = min(min(c0 + a.c.chunk, a.r), u1);
                uint64_t l0 = 0, l1 = 0;
                int64_t h0 = 0, h1 = 0;
                limb_mac2(xcol, m0, m1, lo, hi, l0, h0, l1, h1);
                const int64_t r0 = double_red_words(l0, h0, dm.n[j], dm.ninv[j]);
                v0 = first ? r0 : wadd(v0, r0);
                if (two) {
                    const int64_t r1 = double_red_words(l1, h1, dm.n[j + 1], dm.ninv[j + 1]);
                    v1 = first ? r1 : wadd(v1, r1);
                }
                first = false;
            }
        }
        bconv_store<SUB>(a, dm, b, j, q, v0, dstp + j * a.dst.s1, old0);
        if (two) bconv_store<SUB>(a, dm, b, j + 1, q, v1, dstp + (j + 1) * a.dst.s1, old1);
    }
}

/// dst[i,j,k,l] = src[i,j,p2[k],p3[l]]
__global__ void __launch_bounds__(256) galois_kernel(KView d, KView s, const uint32_t* p2, const uint32_t* p3,
                                                     int64_t lines, int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, r = line / d.n2;
        int64_t j = r % d.n1, i = r / d.n1;
        *kat<int64_t>(d, i, j, k, l) = *kat<int64_t>(s, i, j, p2[k], p3[l]);
    }
}

// Asynchronous global -> shared copies (cp.async): a thread's copies complete in the order of its
// commit groups, and wait_group N returns once at most N of its groups are still in flight.
__device__ __forceinline__ void cp_async8(int64_t* smem, const int64_t* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

struct KsArgs {
    KView parts[HC_MAX_TERMS];  // [B, r, dl, dk] digit t of each of the B ciphertexts (row stride: s0)
    KView keys[HC_MAX_TERMS];   // [2, r, dl, dk] key t restricted to the ciphertext base
    int nterms;
    int64_t batch;              // B; output rows 2i, 2i+1 and summand rows i belong to ciphertext i
    KView add0, add1;  // optional (has_add*) CRT-basis summands of rows 0 / 1, multiplied by mont(1)
    int has_add0, has_add1;
    int full0, full1;  // rows needing the full double reduction
    KView dst;         // [2B, r, dl, dk]
    // optional Galois permutation applied to parts and summands (apply_galois fused into the
    // read, src/bfv.rs:819-820); null means identity
    const uint32_t* p2;
    const uint32_t* p3;
    // tiles in reverse order: a launch that follows one over the same parts and summands starts
    // on the tiles that launch read last, which are still in L2
    int reverse;
};

__device__ __forceinline__ int64_t finish_wide(i128 acc, bool full, const KMods& m, int j) {
    return full ? to_mont64(double_red128(acc, m.n[j], m.ninv[j]), m.n[j], m.ninv[j], m.r2[j])
                : red128(acc, m.n[j], m.ninv[j]);
}

__global__ void __launch_bounds__(256) keyswitch1_kernel(KsArgs a, KMods m, const int64_t* one, int64_t lines,
                                                        int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;  // (j, k)
        int64_t l = (tile - line * chunks) * blockDim.x + threadIdx.x;
        if (l >= a.dst.n3) continue;
        int64_t k = line % a.dst.n2, r = line / a.dst.n2;
        int64_t j = r % a.dst.n1, i = r / a.dst.n1;
        const int64_t sk = a.p2 ? (int64_t)a.p2[k] : k, sl = a.p3 ? (int64_t)a.p3[l] : l;
        i128 acc0 = 0, acc1 = 0;
        for (int t = 0; t < a.nterms; t++) {
            int64_t x = *kat<int64_t>(a.parts[t], i, j, sk, sl);
            int64_t k0 = *kat<int64_t>(a.keys[t], 0, j, k, l);
            int64_t k1 = *kat<int64_t>(a.keys[t], 1, j, k, l);
            acc0 = (i128)((u128)acc0 + (u128)((i128)x * (i128)k0));
            acc1 = (i128)((u128)acc1 + (u128)((i128)x * (i128)k1));
        }
        const int64_t o = one[j];
        if (a.has_add0) acc0 = (i128)((u128)acc0 + (u128)((i128)*kat<int64_t>(a.add0, i, j, sk, sl) * (i128)o));
        if (a.has_add1) acc1 = (i128)((u128)acc1 + (u128)((i128)*kat<int64_t>(a.add1, i, j, sk, sl) * (i128)o));
        *kat<int64_t>(a.dst, 2 * i, j, k, l) = finish_wide(acc0, a.full0, m, (int)j);
        *kat<int64_t>(a.dst, 2 * i + 1, j, k, l) = finish_wide(acc1, a.full1, m, (int)j);
    }
}

/// The key-switch inner product with two adjacent positions l, l + 1 per thread: the keys and the
/// output are read and written as 16-byte pairs (dimension 3 is contiguous and even), the parts
/// and summands gathered singly (through the automorphism's permutation when one is fused). The
/// terms' reads (the two digit words and the two key pairs of each gadget digit) are staged
/// through shared memory by asynchronous copies, KS_STAGES digits ahead of the products, so that
/// the reads in flight do not occupy registers; each thread copies and reads only its own slots
/// (no barrier). Tiles run as ((j, k), chunk, i) with the ciphertext index innermost: the B tiles
/// that read one block of the key are adjacent, so the key comes from DRAM once and B - 1 reads
/// hit L2.
/// COMMON: every term's digit view shares the strides of parts[0] and every key view those of
/// keys[0] (the layouts the ring layer passes), so each thread forms its offsets once and a term's
/// addresses are one addition each.
constexpr int KS_STAGES = 3;

template <bool COMMON>
__global__ void __launch_bounds__(256, 4) keyswitch_async_kernel(KsArgs a, KMods m, const int64_t* one,
                                                                 int64_t lines, int chunks) {
    __shared__ int64_t sx[KS_STAGES][2][256];
    __shared__ longlong2 skey[KS_STAGES][2][256];
    const int tid = threadIdx.x;
    const int64_t tiles = lines * chunks;
    for (int64_t t0 = blockIdx.x; t0 < tiles; t0 += gridDim.x) {
        const int64_t tile = a.reverse ? tiles - 1 - t0 : t0;
        const int64_t i = tile % a.batch, u = tile / a.batch;
        const int64_t line = u / chunks;  // (j, k)
        const int64_t l = 2 * ((u - line * chunks) * blockDim.x + tid);
        if (l >= a.dst.n3) continue;
        const int64_t k = line % a.dst.n2, j = line / a.dst.n2;
        const int64_t sk = a.p2 ? (int64_t)a.p2[k] : k;
        const int64_t sl0 = a.p3 ? (int64_t)a.p3[l] : l, sl1 = a.p3 ? (int64_t)a.p3[l + 1] : l + 1;
        // COMMON offsets (in words) of this thread's digit words and key pairs within every term
        const KView& P = a.parts[0];
        const KView& K = a.keys[0];
        const int64_t po = i * P.s0 + j * P.s1 + sk * P.s2, po0 = po + (P.b3 ? 0 : sl0), po1 = po + (P.b3 ? 0 : sl1);
        const int64_t ko0 = j * K.s1 + k * K.s2 + l, ko1 = ko0 + K.s0;
        auto issue = [&](int t) {
            if (t < a.nterms) {
                const int s = t % KS_STAGES;
                if (COMMON) {
                    const int64_t* pp = reinterpret_cast<const int64_t*>(a.parts[t].p);
                    const int64_t* kp = reinterpret_cast<const int64_t*>(a.keys[t].p);
                    cp_async8(&sx[s][0][tid], pp + po0);
                    cp_async8(&sx[s][1][tid], pp + po1);
                    cp_async16(&skey[s][0][tid], kp + ko0);
                    cp_async16(&skey[s][1][tid], kp + ko1);
                } else {
                    cp_async8(&sx[s][0][tid], kat<int64_t>(a.parts[t], i, j, sk, sl0));
                    cp_async8(&sx[s][1][tid], kat<int64_t>(a.parts[t], i, j, sk, sl1));
                    cp_async16(&skey[s][0][tid], kat<int64_t>(a.keys[t], 0, j, k, l));
                    cp_async16(&skey[s][1][tid], kat<int64_t>(a.keys[t], 1, j, k, l));
                }
            }
            cp_async_commit();  // an empty group past the end keeps the count uniform
        };
#pragma unroll
        for (int t = 0; t < KS_STAGES - 1; t++) issue(t);
        i128 acc00 = 0, acc01 = 0, acc10 = 0, acc11 = 0;  // acc<row><position>
        for (int t = 0; t < a.nterms; t++) {
            issue(t + KS_STAGES - 1);
            cp_async_wait<KS_STAGES - 1>();  // digit t's group has landed
            const int s = t % KS_STAGES;
            const int64_t x0 = sx[s][0][tid], x1 = sx[s][1][tid];
            const longlong2 k0 = skey[s][0][tid], k1 = skey[s][1][tid];
            acc00 = (i128)((u128)acc00 + (u128)((i128)x0 * (i128)k0.x));
            acc01 = (i128)((u128)acc01 + (u128)((i128)x1 * (i128)k0.y));
            acc10 = (i128)((u128)acc10 + (u128)((i128)x0 * (i128)k1.x));
            acc11 = (i128)((u128)acc11 + (u128)((i128)x1 * (i128)k1.y));
        }
        cp_async_wait<0>();
        const int64_t o = one[j];
        if (a.has_add0) {
            acc00 = (i128)((u128)acc00 + (u128)((i128)*kat<int64_t>(a.add0, i, j, sk, sl0) * (i128)o));
            acc01 = (i128)((u128)acc01 + (u128)((i128)*kat<int64_t>(a.add0, i, j, sk, sl1) * (i128)o));
        }
        if (a.has_add1) {
            acc10 = (i128)((u128)acc10 + (u128)((i128)*kat<int64_t>(a.add1, i, j, sk, sl0) * (i128)o));
            acc11 = (i128)((u128)acc11 + (u128)((i128)*kat<int64_t>(a.add1, i, j, sk, sl1) * (i128)o));
        }
        longlong2 w0, w1;
        w0.x = finish_wide(acc00, a.full0, m, (int)j), w0.y = finish_wide(acc01, a.full0, m, (int)j);
        w1.x = finish_wide(acc10, a.full1, m, (int)j), w1.y = finish_wide(acc11, a.full1, m, (int)j);
        *reinterpret_cast<longlong2*>(kat<int64_t>(a.dst, 2 * i, j, k, l)) = w0;
        *reinterpret_cast<longlong2*>(kat<int64_t>(a.dst, 2 * i + 1, j, k, l)) = w1;
    }
}

/// W consecutive words at p (W = 2: one 16-byte access; p must be 16-byte aligned).
template <int W>
__device__ __forceinline__ void load_words(const int64_t* p, int64_t (&v)[W]) {
    if constexpr (W == 2) {
        const longlong2 t = *reinterpret_cast<const longlong2*>(p);
        v[0] = t.x, v[1] = t.y;
    } else {
        v[0] = *p;
    }
}
template <int W>
__device__ __forceinline__ void store_words(int64_t* p, const int64_t (&v)[W]) {
    if constexpr (W == 2) {
        longlong2 t;
        t.x = v[0], t.y = v[1];
        *reinterpret_cast<longlong2*>(p) = t;
    } else {
        *p = v[0];
    }
}

/// (l0 r0, l0 r1 + l1 r0, l1 r1) of B pairs of 2-row ciphertext tensors ([2B, ...] each),
/// reduced per row into [3B, ...]: rows 2i and 2i + 1 receive the first two components of pair i,
/// row 2B + i the third. Each operand comes in two parts along the RNS dimension: rows j < rsplit
/// from *_lo, rows j >= rsplit from *_hi (row j - rsplit). W adjacent positions per thread (W = 2
/// needs an even dimension 3 and 16-byte aligned rows in every view).
template <int W>
__global__ void __launch_bounds__(256) tensor_kernel(KView d, KView lhs_lo, KView lhs_hi, KView rhs_lo, KView rhs_hi,
                                                     int rsplit, KMods m, int full0, int full1, int full2,
                                                     int64_t lines, int chunks) {
    const int64_t tiles = lines * chunks;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        int64_t line = tile / chunks;  // (i, j, k)
        int64_t l = W * ((tile - line * chunks) * blockDim.x + threadIdx.x);
        if (l >= d.n3) continue;
        int64_t k = line % d.n2, r = line / d.n2;
        int64_t j = r % d.n1, i = r / d.n1;
        const bool lo = j < rsplit;
        const int64_t js = lo ? j : j - rsplit;
        const int64_t* lp = lo ? kat<int64_t>(lhs_lo, 2 * i, js, k, l) : kat<int64_t>(lhs_hi, 2 * i, js, k, l);
        const int64_t* rp = lo ? kat<int64_t>(rhs_lo, 2 * i, js, k, l) : kat<int64_t>(rhs_hi, 2 * i, js, k, l);
        const int64_t ls = lo ? lhs_lo.s0 : lhs_hi.s0, rs = lo ? rhs_lo.s0 : rhs_hi.s0;
        int64_t l0[W], l1[W], r0[W], r1[W], o0[W], o1[W], o2[W];
        load_words<W>(lp, l0), load_words<W>(lp + ls, l1);
        load_words<W>(rp, r0), load_words<W>(rp + rs, r1);
#pragma unroll
        for (int w = 0; w < W; w++) {
            const i128 a0 = (i128)l0[w] * (i128)r0[w];
            const i128 a1 = (i128)((u128)((i128)l0[w] * (i128)r1[w]) + (u128)((i128)l1[w] * (i128)r0[w]));
            const i128 a2 = (i128)l1[w] * (i128)r1[w];
            o0[w] = finish_wide(a0, full0, m, (int)j);
            o1[w] = finish_wide(a1, full1, m, (int)j);
            o2[w] = finish_wide(a2, full2, m, (int)j);
        }
        const int64_t B = d.n0 / 3;
        store_words<W>(kat<int64_t>(d, 2 * i, j, k, l), o0);
        store_words<W>(kat<int64_t>(d, 2 * i + 1, j, k, l), o1);
        store_words<W>(kat<int64_t>(d, 2 * B + i, j, k, l), o2);
    }
}

/// One giant step of the homomorphic CRT transform: output digit o (rows 2o, 2o + 1 of dst) is
/// sum over the baby steps j and input digits i of baby(j, i) * L(coef_j, o - i), plus the carried
/// digit o through mont(1), reduced. Each thread holds the accumulators of up to GIANT_OUT output
/// digits, so every baby-step digit is read once for all the outputs it feeds.
constexpr int GIANT_OUT = 4;
constexpr int GIANT_MAX_BABY = 256;

struct GiantArgs {
    KView babies;   // [nbaby * 2d, r, dl, dk]: block j holds sigma^j of the d input digits (rows 2i, 2i + 1)
    KView lcoef;    // [nt, r, dl, 1]: balanced digits of the L' coefficients (CRT basis), broadcast on dim 3
    int nbaby, d;
    short lfirst[GIANT_MAX_BABY];  // row in lcoef of digit 0 of baby j's coefficient
    short lcount[GIANT_MAX_BABY];  // its digit count
    int out0, nout;                // output digits [out0, out0 + nout) of this launch (nout <= GIANT_OUT)
    KView add;                     // the carried digits [2 nadd, ...] (through mont(1))
    int nadd;
    unsigned full;                 // bit o - out0: output digit o needs the full double reduction
    KView dst;                     // [2 used, ...]
};

/// The lcoef values of a tile's line (j, k) are the same for all its positions: the CTA stages
/// them in shared memory once per tile (nt words, dynamic shared memory, after the staging
/// buffers). The (baby step, input digit) units that feed an output digit of the launch are listed
/// by the host (`units`, in giant step order); each thread copies its positions' two words of the
/// next GIANT_STAGES - 1 units into shared memory with cp.async while it multiplies the current
/// one, so that its loads in flight take no registers, and forms every address from one base
/// offset and the row stride. Each thread copies and reads only its own slots.
constexpr int GIANT_STAGES = 4;
constexpr int GIANT_MAX_UNITS = 1024;

/// The (baby step j, input digit i) units of one launch, prepared on the host: the unit's first
/// row in the baby-step tensor (2 d j + 2 i), the output digits o it feeds (bit o of the mask: 0 <=
/// out0 + o - i < lcount[j]) and the coefficient-digit row of output 0 (lfirst[j] + out0 - i;
/// output o reads row fb + o).
struct GiantUnits {
    unsigned int w[GIANT_MAX_UNITS];  // row | mask << 16
    short fb[GIANT_MAX_UNITS];
    int n;
};

__global__ void __launch_bounds__(256) giant_kernel(GiantArgs a, GiantUnits un, KMods m, const int64_t* one,
                                                    int64_t lines, int chunks) {
    extern __shared__ int64_t gsm[];  // [GIANT_STAGES][2][256] staging, then the tile's lcoef
    int64_t* slc = gsm + GIANT_STAGES * 2 * 256;
    const int64_t tiles = lines * chunks;
    const int nt = (int)a.lcoef.n0;
    const int tid = threadIdx.x;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t line = tile / chunks;  // (j, k)
        const int64_t l = (tile - line * chunks) * blockDim.x + tid;
        const int64_t k = line % a.dst.n2, j = line / a.dst.n2;
        __syncthreads();  // the previous tile's readers of slc are done
        for (int t = tid; t < nt; t += blockDim.x) slc[t] = *kat<int64_t>(a.lcoef, t, j, k, 0);
        __syncthreads();
        if (l >= a.dst.n3) continue;
        const int64_t rs = a.babies.s0;  // row stride of the baby-step tensor
        const int64_t* xb = kat<int64_t>(a.babies, 0, j, k, l);
        auto issue = [&](int u) {
            if (u < un.n) {
                const int64_t* xr = xb + (int64_t)(un.w[u] & 0xffff) * rs;
                int64_t* slot = gsm + (u % GIANT_STAGES) * 512;
                cp_async8(slot + tid, xr);
                cp_async8(slot + 256 + tid, xr + rs);
            }
            cp_async_commit();  // an empty group past the end keeps the count uniform
        };
#pragma unroll
        for (int u = 0; u < GIANT_STAGES - 1; u++) issue(u);
        i128 acc0[GIANT_OUT], acc1[GIANT_OUT];
#pragma unroll
        for (int o = 0; o < GIANT_OUT; o++) acc0[o] = acc1[o] = 0;
        for (int u = 0; u < un.n; u++) {
            issue(u + GIANT_STAGES - 1);
            cp_async_wait<GIANT_STAGES - 1>();  // unit u's words have landed
            const unsigned mask = un.w[u] >> 16;
            const int fb = un.fb[u];
            const int64_t* slot = gsm + (u % GIANT_STAGES) * 512;
            const int64_t x0 = slot[tid], x1 = slot[256 + tid];
#pragma unroll
            for (int o = 0; o < GIANT_OUT; o++) {
                if ((mask >> o) & 1) {
                    const int64_t f = slc[fb + o];
                    acc0[o] = (i128)((u128)acc0[o] + (u128)((i128)x0 * (i128)f));
                    acc1[o] = (i128)((u128)acc1[o] + (u128)((i128)x1 * (i128)f));
                }
            }
        }
        cp_async_wait<0>();
#pragma unroll
        for (int o = 0; o < GIANT_OUT; o++) {
            if (o >= a.nout) break;
            const int od = a.out0 + o;
            if (od < a.nadd) {
                const int64_t on = one[j];
                acc0[o] = (i128)((u128)acc0[o] + (u128)((i128)*kat<int64_t>(a.add, 2 * od, j, k, l) * (i128)on));
                acc1[o] = (i128)((u128)acc1[o] + (u128)((i128)*kat<int64_t>(a.add, 2 * od + 1, j, k, l) * (i128)on));
            }
            const bool full = (a.full >> o) & 1;
            *kat<int64_t>(a.dst, 2 * od, j, k, l) = finish_wide(acc0[o], full, m, (int)j);
            *kat<int64_t>(a.dst, 2 * od + 1, j, k, l) = finish_wide(acc1[o], full, m, (int)j);
        }
    }
}

void grid_lines(hc_context ctx, int64_t n3, int64_t lines, int* chunks, unsigned* blocks) {
    *chunks = (int)((n3 + 255) / 256);
    int64_t tiles = lines * *chunks;
    int64_t cap = (int64_t)hc::num_sms(ctx) * 32;
    *blocks = (unsigned)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

}  // namespace

namespace hc {

hc_status launch_bconv_fused(hc_context ctx, const KView& src, const KView& dst, const BconvConsts& c, int r, int rd,
                             int nb, const KMods& sm, const KMods& dm, int64_t ns, const int64_t* sub_mul) {
    BconvArgs a;
    a.src = src;
    a.dst = dst;
    a.c = c;
    a.r = r, a.rd = rd, a.nb = nb;
    a.sub_mul = sub_mul;
    a.npos = src.n2 * src.n3;
    if (a.npos == 0 || ns == 0 || rd == 0) return HC_OK;
    size_t smem = (size_t)r * BCONV_THREADS * 8;
    if (smem > 49152) {
        if (smem > max_smem_optin(ctx)) return fail(HC_ERR_UNSUPPORTED, "base conversion: too many source rows");
        for (auto kern : {bconv_fused_kernel<true, false>, bconv_fused_kernel<true, true>,
                          bconv_fused_kernel<false, false>, bconv_fused_kernel<false, true>}) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_check(e, "bconv smem attribute");
        }
    }
    if (ns * nb > 65535) return fail(HC_ERR_UNSUPPORTED, "base conversion: batch too large");
    // split the outputs over CTAs while the grid is below about two waves of 8 CTAs per SM
    // (each split recomputes the block's lifts and correction, a small part of the work)
    const int64_t cols = (a.npos + BCONV_THREADS - 1) / BCONV_THREADS, base_ctas = cols * ns * nb;
    const int64_t target = (int64_t)num_sms(ctx) * 16;
    int splits = (int)std::min<int64_t>((target + base_ctas - 1) / base_ctas, (rd + 1) / 2);
    splits = std::max(splits, 1);
    a.ochunk = 2 * ((rd + 2 * splits - 1) / (2 * splits));
    splits = (rd + a.ochunk - 1) / a.ochunk;
    dim3 grid((unsigned)cols, (unsigned)(ns * nb), (unsigned)splits);
    const bool one_chunk = c.chunk >= r, sub = sub_mul != nullptr;
    auto kern = one_chunk ? (sub ? bconv_fused_kernel<true, true> : bconv_fused_kernel<true, false>)
                          : (sub ? bconv_fused_kernel<false, true> : bconv_fused_kernel<false, false>);
    kern<<<grid, BCONV_THREADS, smem, stream_of(ctx)>>>(a, sm, dm);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "bconv kernel launch");
}

hc_status launch_galois(hc_context ctx, const KView& d, const KView& s, const uint32_t* p2, const uint32_t* p3) {
    int64_t lines = d.n0 * d.n1 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    int chunks;
    unsigned blocks;
    grid_lines(ctx, d.n3, lines, &chunks, &blocks);
    galois_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(d, s, p2, p3, lines, chunks);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "galois kernel launch");
}

hc_status launch_keyswitch(hc_context ctx, const KView* parts, const KView* keys, int nterms, const KView* add0,
                           const KView* add1, int full0, int full1, const KView& dst, const KMods& m,
                           const int64_t* one_dev, const uint32_t* p2, const uint32_t* p3, bool reverse) {
    if (nterms > HC_MAX_TERMS) return fail(HC_ERR_UNSUPPORTED, "too many gadget digits");
    KsArgs a;
    a.reverse = reverse;
    for (int t = 0; t < nterms; t++) a.parts[t] = parts[t], a.keys[t] = keys[t];
    a.nterms = nterms;
    a.has_add0 = add0 != nullptr;
    a.has_add1 = add1 != nullptr;
    if (add0) a.add0 = *add0;
    if (add1) a.add1 = *add1;
    a.full0 = full0, a.full1 = full1;
    a.dst = dst;
    a.p2 = p2, a.p3 = p3;
    a.batch = dst.n0 / 2;
    int64_t lines = a.batch * dst.n1 * dst.n2;
    if (lines == 0 || dst.n3 == 0) return HC_OK;
    // the paired kernel needs an even dimension 3 and 16-byte aligned key and output rows
    auto aligned = [](const KView& v) {
        return ((uintptr_t)v.p % 16) == 0 && v.s0 % 2 == 0 && v.s1 % 2 == 0 && v.s2 % 2 == 0 && !v.b3;
    };
    bool pair = dst.n3 % 2 == 0 && aligned(dst);
    for (int t = 0; t < nterms; t++) pair = pair && aligned(keys[t]);
    int chunks;
    unsigned blocks;
    if (!pair) {
        grid_lines(ctx, dst.n3, lines, &chunks, &blocks);
        keyswitch1_kernel<<<blocks, 256, 0, stream_of(ctx)>>>(a, m, one_dev, lines, chunks);
        count_launch(ctx);
        return cuda_check(cudaGetLastError(), "keyswitch kernel launch");
    }
    grid_lines(ctx, dst.n3 / 2, lines, &chunks, &blocks);
    bool common = true;
    for (int t = 1; t < nterms; t++) {
        const KView &p = parts[t], &p0 = parts[0], &k = keys[t], &k0 = keys[0];
        common = common && p.s0 == p0.s0 && p.s1 == p0.s1 && p.s2 == p0.s2 && p.b3 == p0.b3 && k.s0 == k0.s0 &&
                 k.s1 == k0.s1 && k.s2 == k0.s2;
    }
    if (common) keyswitch_async_kernel<true><<<blocks, 256, 0, stream_of(ctx)>>>(a, m, one_dev, lines, chunks);
    else keyswitch_async_kernel<false><<<blocks, 256, 0, stream_of(ctx)>>>(a, m, one_dev, lines, chunks);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "keyswitch kernel launch");
}

hc_status launch_giant(hc_context ctx, const KView& babies, const KView& lcoef, int nbaby, int d, const int* lfirst,
                       const int* lcount, const KView* add, int nadd, const unsigned char* full, int used,
                       const KView& dst, const KMods& m, const int64_t* one_dev) {
    if (nbaby > GIANT_MAX_BABY) return fail(HC_ERR_UNSUPPORTED, "too many baby steps");
    int64_t lines = dst.n1 * dst.n2;
    if (lines == 0 || dst.n3 == 0 || used == 0) return HC_OK;
    GiantArgs a;
    a.babies = babies;
    a.lcoef = lcoef;
    a.lcoef.b3 = 1;  // broadcast along dimension 3
    a.nbaby = nbaby, a.d = d;
    for (int j = 0; j < nbaby; j++) {
        if (lfirst[j] > 32767 || lcount[j] > 32767) return fail(HC_ERR_UNSUPPORTED, "too many coefficient digits");
        a.lfirst[j] = (short)lfirst[j], a.lcount[j] = (short)lcount[j];
    }
    a.nadd = add ? nadd : 0;
    if (add) a.add = *add;
    a.dst = dst;
    int chunks;
    unsigned blocks;
    grid_lines(ctx, dst.n3, lines, &chunks, &blocks);
    // the staging buffers and the tile's lcoef words
    const size_t smem = (size_t)(GIANT_STAGES * 2 * 256 + std::max<int64_t>(lcoef.n0, 1)) * 8;
    if (smem > 49152) return fail(HC_ERR_UNSUPPORTED, "too many coefficient digits");
    if (d >= 64) return fail(HC_ERR_UNSUPPORTED, "too many dBFV digits");
    for (int o0 = 0; o0 < used; o0 += GIANT_OUT) {
        a.out0 = o0;
        a.nout = std::min(GIANT_OUT, used - o0);
        a.full = 0;
        for (int o = 0; o < a.nout; o++) a.full |= (unsigned)(full[o0 + o] != 0) << o;
        GiantUnits un;  // the (baby step, input digit) units that feed an output digit of this launch
        un.n = 0;
        for (int bj = 0; bj < nbaby; bj++)
            for (int i = 0; i < d; i++) {
                unsigned mask = 0;
                for (int o = 0; o < a.nout; o++) {
                    const int jj = a.out0 + o - i;
                    if (jj >= 0 && jj < lcount[bj]) mask |= 1u << o;
                }
                if (!mask) continue;
                const int row = bj * 2 * d + 2 * i, fb = lfirst[bj] + a.out0 - i;
                if (un.n == GIANT_MAX_UNITS || row > 0xffff || fb < -32768 || fb > 32767)
                    return fail(HC_ERR_UNSUPPORTED, "too many baby-step units");
                un.w[un.n] = (unsigned)row | (mask << 16);
                un.fb[un.n++] = (short)fb;
            }
        giant_kernel<<<blocks, 256, smem, stream_of(ctx)>>>(a, un, m, one_dev, lines, chunks);
        count_launch(ctx);
        hc_status st = cuda_check(cudaGetLastError(), "giant-step kernel launch");
        if (st) return st;
    }
    return HC_OK;
}

hc_status launch_tensor(hc_context ctx, const KView& d, const KView& lhs_lo, const KView& lhs_hi, const KView& rhs_lo,
                        const KView& rhs_hi, int rsplit, const KMods& m, int f0, int f1, int f2) {
    int64_t lines = (d.n0 / 3) * d.n1 * d.n2;
    if (lines == 0 || d.n3 == 0) return HC_OK;
    // two adjacent positions per thread where every view allows 16-byte accesses
    auto aligned = [](const KView& v) {
        return ((uintptr_t)v.p % 16) == 0 && v.s0 % 2 == 0 && v.s1 % 2 == 0 && v.s2 % 2 == 0 && !v.b3;
    };
    const bool pair = d.n3 % 2 == 0 && aligned(d) && aligned(lhs_lo) && aligned(lhs_hi) && aligned(rhs_lo) &&
                      aligned(rhs_hi);
    int chunks;
    unsigned blocks;
    if (pair) {
        grid_lines(ctx, d.n3 / 2, lines, &chunks, &blocks);
        tensor_kernel<2><<<blocks, 256, 0, stream_of(ctx)>>>(d, lhs_lo, lhs_hi, rhs_lo, rhs_hi, rsplit, m, f0, f1, f2,
                                                              lines, chunks);
    } else {
        grid_lines(ctx, d.n3, lines, &chunks, &blocks);
        tensor_kernel<1><<<blocks, 256, 0, stream_of(ctx)>>>(d, lhs_lo, lhs_hi, rhs_lo, rhs_hi, rsplit, m, f0, f1, f2,
                                                              lines, chunks);
    }
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "tensor kernel launch");
}

}  // namespace hc
