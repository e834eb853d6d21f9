// Shared definitions of the sm_103a ring-arithmetic backend: tensor views as kernels see them,
// exact 64/128-bit modular arithmetic, and launch helpers.
//
// The arithmetic reproduces the reference's integer formulas exactly (same inputs -> same
// representatives), because downstream base-conversion corrections depend on the
// representative, not only on the residue:
//   Barrett multiplication by a constant   cyclosubfield-dbfv/src/hal/ntt.rs:126-158
//   Montgomery reductions (R = 2^64)       cyclosubfield-dbfv/src/hal/mont.rs:36-76
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/halcuda.h"
#include "../../include/ringcuda.h"

typedef __int128 i128;
typedef unsigned __int128 u128;

#define HC_MAX_MODS 96     // RNS rows per call whose moduli travel as kernel parameters
#define HC_MAX_TERMS 64    // inner-product terms per call
#define HC_MAX_STAGES 40   // NTT stages per plan (2^40-point transforms)

// ------------------------------------------------------------------------------------------
// Views
// ------------------------------------------------------------------------------------------

/// A kernel-side 4-D view: shape plus element strides; `s3` is implicitly 1. Broadcast
/// sources carry stride 0 in the broadcast dimensions (`b3` marks a broadcast dimension 3).
struct KView {
    char* p;
    int64_t n0, n1, n2, n3;
    int64_t s0, s1, s2;
    int32_t b3;
};

template <typename T>
__device__ __forceinline__ T* kat(const KView& v, int64_t i, int64_t j, int64_t k, int64_t l) {
    return reinterpret_cast<T*>(v.p) + i * v.s0 + j * v.s1 + k * v.s2 + (v.b3 ? 0 : l);
}

/// Device tables of one base conversion (built by the ring layer; bconv_fused_kernel reads them).
struct BconvConsts {
    const int64_t* qinv;   // [r] plain lifts of (Q_b / p_u)^-1 mod p_u, Montgomery factors
    const int64_t* qinvp;  // [r] qinv[u] * (-p_u^-1) mod 2^64
    const int64_t* mat;    // [nb][rd + 1][r] conversion matrix; row rd of each block: correction row
    const int4* mat3;      // [nb][rd][r] rows 0..rd-1 as limbs (m mod 2^29, m >> 29, their sum, 0)
    const int64_t* qmodp;  // [nb][rd]
    const int64_t* qtab;   // [nb][rd][2 qhalf + 1] mul_mont(q, qmodp) for |q| <= qhalf
    const int64_t* r2p;    // [rd] (R^2 mod p_j) * (-p_j^-1) mod 2^64
    const int32_t* ucol;   // [nb][2] source column range of output block b
    int qhalf;
    int corr_limb;         // the correction row fits the limb products
    int shift;             // log2 of the correction's fixed-point scale
    int chunk;             // acc_before_reduce of the reference
};

/// Montgomery moduli of one call, by value in the kernel's parameter space.
struct KMods {
    int64_t n[HC_MAX_MODS];
    int64_t ninv[HC_MAX_MODS];
    int64_t r2[HC_MAX_MODS];
    int64_t r3[HC_MAX_MODS];
};

// ------------------------------------------------------------------------------------------
// Exact arithmetic
// ------------------------------------------------------------------------------------------

__device__ __forceinline__ int64_t wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
__device__ __forceinline__ int64_t wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }

/// The Barrett quotient q = floor((u x + 2^63) / 2^64) of signed u, x.
/// The high word of the unsigned 128-bit product U X is accumulated from 32-bit limbs with one
/// carry chain; the signed product follows from u x = U X - 2^64 ([u < 0] X + [x < 0] U), and the
/// rounding bit of "+ 2^63" is bit 63 of the low word (bit 31 of its upper limb).
__device__ __forceinline__ uint64_t barrett_q(int64_t u, int64_t x) {
    const uint32_t u0 = (uint32_t)u, u1 = (uint32_t)((uint64_t)u >> 32);
    const uint32_t x0 = (uint32_t)x, x1 = (uint32_t)((uint64_t)x >> 32);
    uint32_t r1, r2, r3;
    asm("{\n\t"
        "mul.hi.u32 %0, %3, %5;\n\t"
        "mad.lo.cc.u32 %0, %3, %6, %0;\n\t"
        "madc.hi.u32 %1, %3, %6, 0;\n\t"
        "mad.lo.cc.u32 %0, %4, %5, %0;\n\t"
        "madc.hi.cc.u32 %1, %4, %5, %1;\n\t"
        "madc.hi.u32 %2, %4, %6, 0;\n\t"
        "mad.lo.cc.u32 %1, %4, %6, %1;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "}"
        : "=&r"(r1), "=&r"(r2), "=&r"(r3)
        : "r"(u0), "r"(u1), "r"(x0), "r"(x1));
    const uint64_t mx = (uint64_t)(x >> 63), mu = (uint64_t)(u >> 63);
    return ((((uint64_t)r3 << 32) | r2) - ((uint64_t)u & mx) - ((uint64_t)x & mu)) + (r1 >> 31);
}

/// Barrett multiplication by the constant (z, u): result z x + q n in wrapping 64-bit arithmetic
/// (|result| <= 3n/4 for |x| <= 2^63), q = barrett_q(u, x).
__device__ __forceinline__ int64_t bmul(int64_t z, int64_t u, int64_t x, int64_t n) {
    return (int64_t)((uint64_t)z * (uint64_t)x + barrett_q(u, x) * (uint64_t)n);
}

/// bmul by the Barrett constant of 1, the reduction step of the lazy transforms: that constant's
/// z is 1 for every odd modulus n >= 3 (1 is its own balanced residue), so z x is x and only the
/// quotient's product remains - the same result as bmul(1, u, x, n) with one product fewer.
__device__ __forceinline__ int64_t bmul1(int64_t u, int64_t x, int64_t n) {
    return (int64_t)((uint64_t)x + barrett_q(u, x) * (uint64_t)n);
}

/// Montgomery reduction of the 128-bit value hi:lo: ((x + m n) >> 64) with m = lo * (-n^-1).
/// The low words of x and m n cancel, so the carry out of the low word is (lo != 0).
__device__ __forceinline__ int64_t red128(uint64_t lo, int64_t hi, int64_t n, int64_t ninv) {
    int64_t m = (int64_t)(lo * (uint64_t)ninv);
    int64_t thi = __mul64hi(m, n);
    return (int64_t)((uint64_t)hi + (uint64_t)thi + (uint64_t)(lo != 0));
}
__device__ __forceinline__ int64_t red128(i128 x, int64_t n, int64_t ninv) {
    return red128((uint64_t)x, (int64_t)(x >> 64), n, ninv);
}

/// Montgomery product of two i64 values (the i128 product must stay within 2^63 n).
__device__ __forceinline__ int64_t mul_mont(int64_t a, int64_t b, int64_t n, int64_t ninv) {
    uint64_t lo = (uint64_t)a * (uint64_t)b;
    int64_t hi = __mul64hi(a, b);
    return red128(lo, hi, n, ninv);
}

/// Double Montgomery reduction of any i128 (x 2^-128 mod n, in [-n, n]).
__device__ __forceinline__ int64_t double_red128(i128 x, int64_t n, int64_t ninv) {
    uint64_t lo = (uint64_t)x;
    int64_t m = (int64_t)(lo * (uint64_t)ninv);
    i128 t = (i128)m * (i128)n;
    i128 carry = (i128)(((u128)lo + (u128)(uint64_t)t) >> 64);
    i128 r1 = (x >> 64) + (t >> 64) + carry;
    return red128(r1, n, ninv);
}

__device__ __forceinline__ int64_t to_mont64(int64_t x, int64_t n, int64_t ninv, int64_t r2) {
    return mul_mont(x, r2, n, ninv);
}
__device__ __forceinline__ int64_t to_mont128(i128 x, int64_t n, int64_t ninv, int64_t r3) {
    return mul_mont(red128(x, n, ninv), r3, n, ninv);
}

/// mul_mont(a, b) for a constant b with bp = b * ninv mod 2^64: the Montgomery quotient
/// m = lo(a b) ninv equals a bp mod 2^64, and lo(a b) != 0 exactly when m != 0 (ninv is odd), so
/// the low word of a b is never formed. The same integers as mul_mont(a, b, n, ninv).
__device__ __forceinline__ int64_t mul_mont_c(int64_t a, int64_t b, int64_t bp, int64_t n) {
    const int64_t m = (int64_t)((uint64_t)a * (uint64_t)bp);
    return (int64_t)((uint64_t)__mul64hi(a, b) + (uint64_t)__mul64hi(m, n) + (uint64_t)(m != 0));
}

/// double_red128 of the 128-bit value hi:lo: the first reduction's carry out of the low word is
/// (lo != 0) (the low words of x and m n cancel), so the low word of m n is never formed.
__device__ __forceinline__ int64_t double_red_words(uint64_t lo, int64_t hi, int64_t n, int64_t ninv) {
    const int64_t m = (int64_t)(lo * (uint64_t)ninv);
    const i128 r1 = (i128)hi + (i128)__mul64hi(m, n) + (i128)(lo != 0);
    return red128((uint64_t)r1, (int64_t)(r1 >> 64), n, ninv);
}

__device__ __forceinline__ i128 ld128(const void* p) {
    longlong2 v = *reinterpret_cast<const longlong2*>(p);
    return (i128)(((u128)(uint64_t)v.y << 64) | (uint64_t)v.x);
}
__device__ __forceinline__ void st128(void* p, i128 x) {
    longlong2 v;
    v.x = (long long)(uint64_t)x;
    v.y = (long long)(x >> 64);
    *reinterpret_cast<longlong2*>(p) = v;
}

// ------------------------------------------------------------------------------------------
// Batched CRT transforms
// ------------------------------------------------------------------------------------------

/// One (ring element, RNS factor) slab of a batched transform: deg_L' rows of deg_K residues.
struct CrtSlab {
    const void* plan2;     // NTT plan along dimension 2 (length deg_L')
    const void* plan3;     // NTT plan along dimension 3 (length deg_K)
    int64_t* data;         // row k at data + k * s2, contiguous
    const int64_t* op;     // operand slab (HC_CRT_MUL), row k at op + k * op_s2
    const int64_t* kl;     // CRT kernel of this factor along dimension 2 (deg_L' entries)
    const int64_t* kk;     // ... along dimension 3 (deg_K entries)
    const int64_t* ikl;    // inverse kernels
    const int64_t* ikk;
    int64_t s2, op_s2;
    int64_t n, ninv;       // Montgomery modulus of the factor
    int32_t dl, dk;
    int32_t ops;           // HC_CRT_* bits
    int32_t shapes;        // specialised kernel shapes: dimension 3 | dimension 2 << 8 (0: generic)
};

/// Launch shape of the persistent batched-transform kernel (chosen by the autotuner).
struct CrtLaunch {
    int threads;      // per CTA
    int ctas_per_sm;  // persistent grid = SMs x this
    int logv;         // dimension-2 tile: 2^logv columns
};

// ------------------------------------------------------------------------------------------
// Host-side helpers shared by the translation units
// ------------------------------------------------------------------------------------------
namespace hc {

void set_error(const std::string& msg);
hc_status fail(hc_status st, const std::string& msg);
hc_status cuda_check(cudaError_t e, const char* what);
cudaStream_t stream_of(hc_context ctx);
void count_launch(hc_context ctx, uint64_t n = 1);
/// Every device or pinned-host allocation call of the library counts itself (hc_memory_stats).
void count_alloc();
uint64_t alloc_calls();
int num_sms(hc_context ctx);
size_t max_smem_optin(hc_context ctx);
int device_of(hc_context ctx);
hc_status intt_mul_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim,
                              hc_view mul, const hc_modulus* mods, size_t nmods);
hc_status ntt_mul_mont64_dim_from(hc_context ctx, hc_view dst, hc_view src, const hc_ntt_plan* plans, size_t nplans,
                                  hc_data_dim dim, hc_view mul, const hc_modulus* mods, size_t nmods);

}  // namespace hc
